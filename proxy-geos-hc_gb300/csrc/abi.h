// abi.h -- internals shared by the C-ABI translation units: error reporting, device
// allocation helpers and the mesh handle.
#pragma once
#include <cuda_runtime.h>

#include <new>
#include <string>

#include "../../include/semgb.h"
#include "host_util.h"
#include "kernels.h"

namespace semgb {
void set_last_error(const std::string &msg);
}  // namespace semgb

inline int sem_fail(int code, const std::string &msg)
{
    semgb::set_last_error(msg);
    return code;
}

#define CUDA_TRY(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return sem_fail(e_ == cudaErrorMemoryAllocation ? SEM_ERR_OOM : SEM_ERR_CUDA,    \
                            std::string(#call) + ": " + cudaGetErrorString(e_));             \
    } while (0)

#define GUARD_BEGIN try {
#define GUARD_END                                                                            \
    }                                                                                        \
    catch (const std::bad_alloc &) { return sem_fail(SEM_ERR_OOM, "host allocation failed"); } \
    catch (...) { return sem_fail(SEM_ERR_STATE, "unexpected exception"); }

template <class T>
inline cudaError_t dalloc(T **p, size_t n)
{
    *p = nullptr;
    if (n == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T));
}

template <class T>
inline void dfree(T *&p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

struct sem_mesh {
    semgb::Box box;
    semgb::Gll gll;
    semgb::Geometry geo;
    int device = 0;
    float *d_vel = nullptr;     // [n_elem]
    float *d_slow2 = nullptr;   // [n_int] when the node model is active (device layout)
    int32_t *d_conn = nullptr;  // [n_elem * npe], built on first use by the element kernel
    uint64_t model_version = 1;
};
