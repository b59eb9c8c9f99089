// fednl_smem.h -- the dynamic shared-memory limit of a kernel is a per-function setting shared by
// every handle in the process: it is only ever raised, so that a handle created later with a
// smaller need does not lower the limit another live handle launches with.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <mutex>

inline cudaError_t fednl_raise_dyn_smem(const void* fn, size_t bytes)
{
    static std::mutex mu;
    static std::map<const void*, size_t> cur;
    std::lock_guard<std::mutex> g(mu);
    size_t& c = cur[fn];
    if (bytes <= c) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) c = bytes;
    return e;
}
