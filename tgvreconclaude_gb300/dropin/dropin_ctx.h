// The drop-in translation units share one tgvg context per process (created
// on first use) and one error-to-exception mapping.
#pragma once
#include <mutex>
#include <stdexcept>
#include <string>

#include "tgvg.h"

inline tgvg_ctx* tgvg_dropin_ctx() {
    static std::once_flag once;
    static tgvg_ctx* c = nullptr;
    static int rc = 0;
    std::call_once(once, [] { rc = tgvg_create(0, &c); });
    if (rc != TGVG_OK) throw std::runtime_error(std::string("tgvg_create: ") + tgvg_strerror(rc));
    return c;
}

inline void tgvg_dropin_check(int rc, const char* what) {
    if (rc != TGVG_OK) {
        std::string msg = std::string(what) + ": " + tgvg_strerror(rc);
        const char* d = tgvg_last_error(tgvg_dropin_ctx());
        if (d && *d) msg += std::string(" (") + d + ")";
        throw std::runtime_error(msg);
    }
}
