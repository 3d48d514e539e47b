/* ref_kernels.cu -- the reference's own GPU kernels, compiled from its source for the reference-GPU comparator
 * (test and measurement infrastructure, never the product).
 *
 * Defines the device macros exactly as the reference's CUDA backend does (src/phygas_cuda.cu:7-13) and includes the
 * reference's kernel header, src/phygas_kernel_body.h (pg_lin_k, pg_chi2_k, pg_finish_k, pg_pair_k), from the
 * reference checkout, with C linkage so that a host program can look the kernels up by name.  Built by
 * `make -C oracle ref-gpu-ptx` with the reference's own device flags (--fmad=false -O3, scripts/build_gpu_server.sh:31)
 * for compute_103a into oracle/_ref/ref_kernels.ptx; oracle/ref_gpu_main.cpp loads it and drives the kernels the
 * way the reference's BOINC app does.  Nothing of the reference is copied: the header is read where it lies.
 */
#define PG_GLOBAL
#define PG_DEVICE __device__ static inline
#define PG_KERNEL __global__
#define PG_TID ((int)(blockIdx.x * blockDim.x + threadIdx.x))
#define PG_U64 unsigned long long
#define PG_LONG long long
#define PG_INF __longlong_as_double(0x7ff0000000000000LL)
extern "C" {
#include "phygas_kernel_body.h"
}
