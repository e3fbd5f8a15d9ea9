/* A host program in plain C that drives the solver through include/tgvg.h only,
 * the way a C, cgo or JNI binding of the reference's tgv_minimize,
 * tgv_minimize_oc and tgv_minimize_streaming (reference src/tgv.hpp) would.
 *
 *   c_abi_host <dir>
 *
 * <dir> holds meta.txt ("n nbins nleaf iters alpha0 alpha1"), cubes.bin
 * (n tgvg_cube records), hists.bin (n * nbins uint32) and leaves.bin (nleaf
 * tgvg_leaf records).  The program solves the problem in the three semantics
 * and writes state_<mode>.bin (n tgvg_state records).  It also checks that an
 * invalid call returns an error code with a message.  Exit status: 0 on
 * success, 2 when the library reports an error (the message goes to stderr). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tgvg.h"

static void* read_all(const char* dir, const char* name, size_t bytes) {
    char path[4096];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    void* p = malloc(bytes ? bytes : 1);
    const size_t got = p ? fread(p, 1, bytes, f) : 0;
    fclose(f);
    if (got != bytes) {
        free(p);
        return NULL;
    }
    return p;
}

static int fail(int rc, const char* what) {
    fprintf(stderr, "%s: %s\n", what, tgvg_strerror(rc));
    return 2;
}

int main(int argc, char** argv) {
    if (argc != 2) {
        fprintf(stderr, "usage: %s <dir>\n", argv[0]);
        return 1;
    }
    const char* dir = argv[1];
    char path[4096];
    snprintf(path, sizeof(path), "%s/meta.txt", dir);
    FILE* m = fopen(path, "r");
    long long n = 0;
    int nbins = 0, nleaf = 0, iters = 0;
    float a0 = 0.f, a1 = 0.f;
    if (!m || fscanf(m, "%lld %d %d %d %f %f", &n, &nbins, &nleaf, &iters, &a0, &a1) != 6) {
        fprintf(stderr, "cannot read %s\n", path);
        return 1;
    }
    fclose(m);
    tgvg_cube* cubes = (tgvg_cube*)read_all(dir, "cubes.bin", sizeof(tgvg_cube) * (size_t)n);
    uint32_t* hists = (uint32_t*)read_all(dir, "hists.bin", sizeof(uint32_t) * (size_t)n * (size_t)nbins);
    tgvg_leaf* leaves = (tgvg_leaf*)read_all(dir, "leaves.bin", sizeof(tgvg_leaf) * (size_t)nleaf);
    tgvg_state* out = (tgvg_state*)malloc(sizeof(tgvg_state) * (size_t)(n ? n : 1));
    if (!cubes || !hists || !leaves || !out) {
        fprintf(stderr, "cannot read the inputs in %s\n", dir);
        return 1;
    }

    tgvg_ctx* ctx = NULL;
    int rc = tgvg_create(0, &ctx);
    if (rc) return fail(rc, "tgvg_create");

    tgvg_params prm;
    memset(&prm, 0, sizeof(prm));
    prm.alpha0 = a0;
    prm.alpha1 = a1;
    prm.iters = iters;
    prm.init = TGVG_INIT_MEDIAN;
    prm.check_every = 10;

    /* an invalid request is refused with a message, and the context stays usable */
    rc = tgvg_tgv_minimize(ctx, cubes, hists, n, 7, leaves, nleaf, TGVG_MODE_INMEM, &prm, NULL, out, NULL);
    if (rc == 0 || strlen(tgvg_strerror(rc)) == 0) {
        fprintf(stderr, "nbins = 7 was accepted\n");
        return 3;
    }

    const int modes[3] = {TGVG_MODE_INMEM, TGVG_MODE_OC, TGVG_MODE_STREAM};
    for (int k = 0; k < 3; ++k) {
        tgvg_stats st;
        rc = tgvg_tgv_minimize(ctx, cubes, hists, n, nbins, leaves, nleaf, modes[k], &prm, NULL, out, &st);
        if (rc) return fail(rc, "tgvg_tgv_minimize");
        snprintf(path, sizeof(path), "%s/state_%d.bin", dir, modes[k]);
        FILE* f = fopen(path, "wb");
        if (!f || fwrite(out, sizeof(tgvg_state), (size_t)n, f) != (size_t)n) {
            fprintf(stderr, "cannot write %s\n", path);
            return 1;
        }
        fclose(f);
        printf("mode %d: %d levels, %lld leaf-iterations\n", modes[k], st.n_levels, (long long)st.leaf_iters);
    }
    rc = tgvg_destroy(ctx);
    if (rc) return fail(rc, "tgvg_destroy");
    free(cubes);
    free(hists);
    free(leaves);
    free(out);
    return 0;
}
