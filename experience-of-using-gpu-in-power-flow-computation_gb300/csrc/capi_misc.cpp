// capi_misc.cpp -- device query used by the command-line driver (the GPU
// banner of initGPU, GPU/sistema.cuh:426-468).
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "gbpf_internal.h"

extern "C" gbpf_status gbpf_device_info(int device, int *count, char *name, size_t name_cap,
                                        int props[6]) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        gbpf::set_error(std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
        return GBPF_E_CUDA;
    }
    if (count) *count = n;
    if (device < 0 || device >= n) return GBPF_E_ARG;
    cudaDeviceProp p;
    e = cudaGetDeviceProperties(&p, device);
    if (e != cudaSuccess) {
        gbpf::set_error(std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e));
        return GBPF_E_CUDA;
    }
    if (name && name_cap) std::snprintf(name, name_cap, "%s", p.name);
    if (props) {
        props[0] = p.major;
        props[1] = p.minor;
        props[2] = p.warpSize;
        props[3] = p.maxThreadsPerMultiProcessor;
        props[4] = p.maxThreadsPerBlock;
        props[5] = p.multiProcessorCount;
    }
    return GBPF_OK;
}
