// ref_shim.h -- TEST INFRASTRUCTURE ONLY.
//
// Lets the reference's CUDA kernel bodies (plain scalar C arithmetic, no
// intrinsics) and its gold host driver compile for the CPU with g++, so the
// reference's own code can produce golden outputs on seeded inputs.  The
// CUDA qualifiers become nothing, the launch built-ins become thread-local
// variables that the emulated launchers in ref_launch.inc set per "thread",
// and the runtime calls the host driver makes become host memory operations.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
using std::abs;
using std::sqrt;

#define __global__
#define __device__
#define __host__
#define __constant__
#define __syncthreads() ((void)0)

struct shim_uint3 { int x, y, z; };
static thread_local shim_uint3 blockIdx, threadIdx, blockDim, gridDim;

typedef int cudaError_t;
#define cudaSuccess 0
enum { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1,
       cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
static inline int cudaMalloc(void** p, size_t n) { *p = calloc(n ? n : 1, 1); return *p ? 0 : 2; }
static inline int cudaFree(void* p) { free(p); return 0; }
static inline int cudaMemset(void* p, int v, size_t n) { memset(p, v, n); return 0; }
static inline int cudaMemcpy(void* d, const void* s, size_t n, int) { memmove(d, s, n); return 0; }
static inline int cudaGetLastError(void) { return 0; }
static inline const char* cudaGetErrorString(int) { return "no error"; }
static inline int cudaThreadSynchronize(void) { return 0; }
static inline int cudaDeviceSynchronize(void) { return 0; }

// The driver prints progress per sub-iteration and calls system("PAUSE") on
// error paths; silence both.
#define printf(...) ((void)0)
#define system(x) 0

// The reference's 4R sub-ray kernel (Tomo_OSTR.cu:1453-1515) reads two batch
// counts that Tomo_OSTR.cu never defines; one batch covers the detector here.
static int nBatchBINSx_4R = 1, nBatchBINSy_4R = 1;
