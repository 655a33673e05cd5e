// Bounds-checked builds.  Compiled with -DTCSEM_CHECK (tcsem_fdtd_gb300/build.py,
// build(check=True): libtcsem_check.so), every global load and store of the kernels at
// a computed index is tested against the extent of its array first; an index outside
// it records TCSEM_CHECK_CODE in the kernel's device error word (the host reports it as
// TCSEM_ERR_CUDA with its own message) and the access is skipped -- nothing traps.
// Without the macro the tests compile to nothing.
#pragma once
#include <cuda_runtime.h>

#define TCSEM_CHECK_CODE 2

#ifdef TCSEM_CHECK
namespace tcsem {
__device__ __forceinline__ bool check_index(long long i, long long n, int *err) {
    if (i >= 0 && i < n) return true;
    if (err) atomicExch(err, TCSEM_CHECK_CODE);
    return false;
}
}  // namespace tcsem
// true when 0 <= i < n; otherwise records the miss in *err
#define TCSEM_IN(i, n, err) ::tcsem::check_index((long long)(i), (long long)(n), (err))
#else
#define TCSEM_IN(i, n, err) true
#endif
