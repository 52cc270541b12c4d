/*
 * ref_shim.h - forced-include header that lets the reference's device source
 * (ptGraph/gpu_kernels.cu) compile as plain host C++ (TEST INFRASTRUCTURE
 * ONLY).
 *
 * The reference's kernels are written against the CUDA execution model:
 * __global__ functions that read threadIdx/blockIdx/blockDim/gridDim through a
 * grid-stride loop (ptGraph/gpu_kernels.cuh:12-24) and update shared values
 * with atomicMin/atomicAdd.  This header supplies host versions of exactly
 * those names: the qualifiers expand to nothing, the four index variables are
 * thread_local globals that oracle/ref_harness.cpp sets before it calls a
 * kernel once per emulated (block, thread), and the atomics are plain
 * read-modify-writes (the emulation is sequential).  No reference source is
 * copied; the recipe in oracle/Makefile compiles the file where it lies.
 */
#ifndef PTG_REF_SHIM_H
#define PTG_REF_SHIM_H

#include <climits>
#include <cstdint>
#include <sys/types.h>

#define __global__
#define __device__
#define __host__

struct ptg_emu_dim3 {
    unsigned int x, y, z;
};

extern thread_local ptg_emu_dim3 threadIdx, blockIdx, blockDim, gridDim;

static inline unsigned int atomicMin(unsigned int *addr, unsigned int val) {
    unsigned int old = *addr;
    if (val < old) *addr = val;
    return old;
}

static inline unsigned int atomicAdd(unsigned int *addr, unsigned int val) {
    unsigned int old = *addr;
    *addr = old + val;
    return old;
}

#endif
