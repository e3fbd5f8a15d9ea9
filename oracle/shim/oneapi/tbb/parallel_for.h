// Serial stand-in for tbb::parallel_for: the body runs once over the whole
// range on the calling thread.  Test infrastructure for the oracle build.
#pragma once
#include "blocked_range.h"

namespace tbb {
template <typename Range, typename Body>
void parallel_for(const Range& r, const Body& body) { body(r); }
}  // namespace tbb
namespace oneapi { namespace tbb { using ::tbb::parallel_for; } }
