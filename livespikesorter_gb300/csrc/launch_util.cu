// launch_util.cu -- process-wide kernel attributes shared by every handle.
//
// A kernel's dynamic shared-memory limit (cudaFuncAttributeMaxDynamicSharedMemorySize) belongs to
// the kernel on a device, not to a launch: when handles of different shapes set it from different
// host threads, one can lower it between another's set and launch, and that launch then fails.
// raise_smem_limit only ever raises it, under one lock, so every launch sized below the
// recorded value stays valid.
#include "lss_kernels.cuh"

#include <map>
#include <mutex>
#include <utility>

namespace lss {

cudaError_t raise_smem_limit(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> limit;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = limit[{kernel, dev}];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    else cudaGetLastError();   // a refused size is reported here, not to the caller's next check
    return e;
}

}  // namespace lss
