// Serial stand-in for the TBB blocked_range used by the reference's Stage-1
// builder.  Test infrastructure for the oracle build; written for this project.
#pragma once
#include <cstddef>

namespace tbb {
template <typename T>
class blocked_range {
public:
    blocked_range(T b, T e, std::size_t grain = 1) : b_(b), e_(e) { (void)grain; }
    T begin() const { return b_; }
    T end() const { return e_; }
    bool empty() const { return !(b_ < e_); }
private:
    T b_, e_;
};
}  // namespace tbb
namespace oneapi { namespace tbb { using ::tbb::blocked_range; } }
