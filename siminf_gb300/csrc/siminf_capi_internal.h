/*
 * siminf_capi_internal.h -- what the translation units behind the C ABI
 * share: the model handle and the argument check and per-thread status of
 * siminf_capi.cpp.
 */
#ifndef SIMINF_CAPI_INTERNAL_H
#define SIMINF_CAPI_INTERNAL_H

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_launch.h"

/* A device model: its name and the launchers of its kernels. */
struct siminf_gpu_model {
    char name[64];
    const siminf::Launchers *L;
};

namespace siminf {

/* The checks siminf_gpu_run_solver_ssm applies to its arguments. */
int capi_validate(const siminf_gpu_solver_args *a, const Launchers *L);

/* Record the calling thread's status (read by siminf_gpu_last_status). */
void capi_set_status(int code, int node, int tr, int evi, double time, double rate,
                     const char *msg);
void capi_clear_status();

/* Record a failed CUDA call; returns SIMINF_GPU_ERR_CUDA. */
int capi_cuda_fail(cudaError_t e, const char *what);

}  // namespace siminf

#endif
