// common.cuh -- shared device helpers of libnrgb300 (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nrgb300.h"

#define NR_API extern "C" __attribute__((visibility("default")))

// Status bits of the device status word kept in the workspace.
#define NR_FLAG_NONFINITE 1
#define NR_FLAG_TIMEOUT 2

namespace nr {

// Geometry as the kernels use it: the caller's nr_geom passed by value
// (__grid_constant__) plus per-launch derived constants.
struct Geo {
    nr_geom g;
    float xmax, ymax, zmax;  // far corner of the volume
};

__host__ inline Geo make_geo(const nr_geom& g) {
    Geo d;
    d.g = g;
    d.xmax = g.x_p0 + (float)g.nx * g.vx;
    d.ymax = g.y_p0 + (float)g.ny * g.vy;
    d.zmax = g.z_p0 + (float)g.nz * g.vz;
    return d;
}

// Source of one view: rotation about the y axis at the origin,
// (R sin t, sourceY, R cos t), Tomo_OSTR.cu:1340-1345.  Evaluated in double
// and rounded once (the reference uses float sinf/cosf; a 2-ulp sine moves the
// source by ~2e-5 mm, which shows up against the FP64 oracle wherever a ray
// grazes a high-contrast edge).  s2 = |source|^2, the SBP depth-weight
// numerator (Tomo_OSTR.cu:1634).  One thread per block computes it.
struct ViewSrc {
    float x0, y0, z0, ct, s2;
};

__device__ __forceinline__ ViewSrc view_source(const nr_geom& g, float theta) {
    double s, c;
    sincos((double)theta, &s, &c);
    ViewSrc v;
    v.x0 = (float)((double)g.sourceR * s);
    v.z0 = (float)((double)g.sourceR * c);
    v.y0 = g.sourceY;
    v.ct = (float)c;
    v.s2 = v.x0 * v.x0 + v.y0 * v.y0 + v.z0 * v.z0;
    return v;
}

// Bin centre on the stationary detector, Tomo_OSTR.cu:1349-1356.  The
// reference forms x_d0 + (i+0.5)*Bsize in double and rounds once to float;
// (i+0.5)*Bsize is exact in double, so one fused multiply-add (single
// rounding of the exact value) reproduces it.
__device__ __forceinline__ float bin_x(const nr_geom& g, int i) {
    return __fmaf_rn((float)i + 0.5f, g.bx, g.x_d0);
}
__device__ __forceinline__ float bin_y(const nr_geom& g, int j) {
    return __fmaf_rn((float)j + 0.5f, g.by, g.y_d0);
}
// Voxel centre, Tomo_OSTR.cu:1624-1626 (same double-then-round form).
__device__ __forceinline__ float vox_x(const nr_geom& g, int i) {
    return __fmaf_rn((float)i + 0.5f, g.vx, g.x_p0);
}
__device__ __forceinline__ float vox_y(const nr_geom& g, int i) {
    return __fmaf_rn((float)i + 0.5f, g.vy, g.y_p0);
}
__device__ __forceinline__ float vox_z(const nr_geom& g, int i) {
    return __fmaf_rn((float)i + 0.5f, g.vz, g.z_p0);
}

__host__ inline bool geom_ok(const nr_geom* g) {
    if (!g) return false;
    if (g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || g->nbx <= 0 || g->nby <= 0 || g->n_angles <= 0)
        return false;
    if (!(g->vx > 0.f) || !(g->vy > 0.f) || !(g->vz > 0.f) || !(g->bx > 0.f) || !(g->by > 0.f))
        return false;
    if ((int64_t)g->nx * g->ny * g->nz >= (int64_t)1 << 31) return false;
    if ((int64_t)g->nbx * g->nby * g->n_angles >= (int64_t)1 << 31) return false;
    return true;
}

__host__ inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

__host__ inline nr_status launch_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NR_OK : NR_ERR_LAUNCH;
}

__host__ inline unsigned cdiv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// A captured launch sequence: the graph and its executable instance (the
// opaque handle of nr_ostr_graph_create / nr_batch_graph_create).
struct GraphHandle {
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

// Ends the capture on s (always), instantiates on success and returns the
// handle in *out; on any failure nothing is left allocated.
__host__ inline nr_status finish_capture(cudaStream_t s, nr_status st, void** out) {
    cudaGraph_t gr = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &gr);
    if (st != NR_OK || ec != cudaSuccess || !gr) {
        if (gr) cudaGraphDestroy(gr);
        cudaGetLastError();
        return st != NR_OK ? st : NR_ERR_CUDA;
    }
    cudaGraphExec_t ex = nullptr;
    if (cudaGraphInstantiate(&ex, gr, 0) != cudaSuccess) {
        cudaGraphDestroy(gr);
        cudaGetLastError();
        return NR_ERR_CUDA;
    }
    *out = new GraphHandle{gr, ex};
    return NR_OK;
}

}  // namespace nr
