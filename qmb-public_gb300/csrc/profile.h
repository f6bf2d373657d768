// Launch counting and per-group kernel timing (see profile.cpp).
#pragma once

#include <cuda_runtime.h>

namespace qmbx {

// kGroupEnumerate is the main term walk; kGroupDiagonal the separate
// passes over diagonal terms that follow it; kGroupSort the radix sorts
// (histogram, scan and scatter passes); kGroupSpmv the products with a
// materialised matrix and the adjoint products formed from a hit log (the
// replay, and the adjoint walk that stands in for an incomplete record,
// launched every time and walking no row when the record is complete)
enum ProfileGroup {
    kGroupEnumerate = 0,
    kGroupKeys = 1,
    kGroupSelect = 2,
    kGroupOther = 3,
    kGroupDiagonal = 4,
    kGroupSort = 5,
    kGroupSpmv = 6,
    kProfileGroups = 7
};

void note_launch(int n);

// Brackets the launches made during its lifetime with events on `stream`
// when profiling is enabled; does nothing otherwise.
class Timing {
   public:
    Timing(int group, cudaStream_t stream);
    ~Timing();
    Timing(const Timing&) = delete;
    Timing& operator=(const Timing&) = delete;

   private:
    int group_;
    cudaStream_t stream_;
    cudaEvent_t start_ = nullptr;
    cudaEvent_t stop_ = nullptr;
};

}  // namespace qmbx

// Launch one kernel (the variadic argument is the launch expression) inside a
// timing scope of the given group and count it.
#define QMBX_KERNEL(group, stream, ...)               \
    do {                                              \
        ::qmbx::Timing qmbx_timing_((group), (stream)); \
        __VA_ARGS__;                                  \
        ::qmbx::note_launch(1);                       \
    } while (0)
