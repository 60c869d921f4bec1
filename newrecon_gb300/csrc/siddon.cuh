// siddon.cuh -- exact-chord-length ray walk through the voxel grid (device).
//
// The Siddon/Jacobs incremental walk of
// rayTrace3D_GPU_direct_notexturememory_OSTR (Tomo_OSTR.cu:612-890), written
// in a drift-free parametrisation: the distance s (mm) from the volume entry
// point, with the k-th crossing of each axis computed as fma(k, step, first)
// instead of a running sum, so crossings keep full float accuracy over
// hundreds of steps (the reference's running sum of alpha increments drifts
// by O(steps) ulps of alpha ~ 1, i.e. up to ~1e-3 mm at clinical sizes).  The
// exit distance is the smallest per-axis exit-plane crossing, computed with
// the same fma, so the walk stops exactly when the first axis would leave the
// grid and every read stays in bounds by construction.
#pragma once

#include "common.cuh"

namespace nr {

#define NR_FINF __int_as_float(0x7f800000)

// min(a, b, c) in one three-input min (sm_100 and later): the walk takes the
// nearest of the three axis crossings once per segment.
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Per-axis walk state.
struct Axis {
    float first;   // distance (mm) from the entry point to the first plane crossed
    float step;    // distance between consecutive planes (mm)
    float last;    // distance to the plane through which the ray leaves the grid
    int idx;       // voxel index at the entry point
    int dir;       // +1 / -1 / 0
};

// e: entry coordinate in voxel units; d: ray direction component; L: ray
// length; n: grid size; v: voxel size.
__device__ __forceinline__ Axis axis_setup(float e, float d, float L, int n, float v) {
    Axis a;
    int i = (int)floorf(e);
    i = max(0, min(n - 1, i));
    a.idx = i;
    if (d == 0.f) {
        a.dir = 0;
        a.first = NR_FINF;
        a.step = NR_FINF;
        a.last = NR_FINF;
        return a;
    }
    a.step = __fdiv_rn(v * L, fabsf(d));
    float f;
    int cnt;
    if (d > 0.f) {
        a.dir = 1;
        f = (float)(i + 1) - e;
        cnt = n - i;
    } else {
        a.dir = -1;
        f = e - (float)i;
        cnt = i + 1;
    }
    a.first = f * a.step;
    a.last = __fmaf_rn((float)(cnt - 1), a.step, a.first);
    return a;
}

// The walk's set-up for the ray (x0,y0,z0) -> (x1,y1,z1): its length L, the
// per-axis state from the volume entry point and the exit distance smax.
// Returns false when the ray misses the volume (the reference's status -1);
// LENGTH_ONLY stops after the slab test with only L set.
struct RayAxes {
    Axis ax, ay, az;
    float smax, L;
};

template <bool LENGTH_ONLY>
__device__ __forceinline__ bool ray_axes(const Geo& G, float x0, float y0, float z0, float x1,
                                         float y1, float z1, RayAxes& R) {
    const nr_geom& g = G.g;
    const float dx = x1 - x0, dy = y1 - y0, dz = z1 - z0;
    const float L = sqrtf(dx * dx + dy * dy + dz * dz);
    if (!(L > 0.f && L < NR_FINF)) return false;
    R.L = L;
    float amin = -NR_FINF, amax = NR_FINF;
    // Parametric slab intersection, Tomo_OSTR.cu:641-726.
    if (dx != 0.f) {
        const float a0 = __fdiv_rn(g.x_p0 - x0, dx), a1 = __fdiv_rn(G.xmax - x0, dx);
        amin = fmaxf(amin, fminf(a0, a1));
        amax = fminf(amax, fmaxf(a0, a1));
    } else if (x0 >= G.xmax || x0 <= g.x_p0) {
        return false;
    }
    if (dy != 0.f) {
        const float a0 = __fdiv_rn(g.y_p0 - y0, dy), a1 = __fdiv_rn(G.ymax - y0, dy);
        amin = fmaxf(amin, fminf(a0, a1));
        amax = fminf(amax, fmaxf(a0, a1));
    } else if (y0 >= G.ymax || y0 <= g.y_p0) {
        return false;
    }
    if (dz != 0.f) {
        const float a0 = __fdiv_rn(g.z_p0 - z0, dz), a1 = __fdiv_rn(G.zmax - z0, dz);
        amin = fmaxf(amin, fminf(a0, a1));
        amax = fminf(amax, fmaxf(a0, a1));
    } else if (z0 >= G.zmax || z0 <= g.z_p0) {
        return false;
    }
    if (!(amin < amax)) return false;
    if (LENGTH_ONLY) return true;
    // Entry point in voxel units.
    const float ex = __fdiv_rn(__fmaf_rn(amin, dx, x0 - g.x_p0), g.vx);
    const float ey = __fdiv_rn(__fmaf_rn(amin, dy, y0 - g.y_p0), g.vy);
    const float ez = __fdiv_rn(__fmaf_rn(amin, dz, z0 - g.z_p0), g.vz);
    R.ax = axis_setup(ex, dx, L, g.nx, g.vx);
    R.ay = axis_setup(ey, dy, L, g.ny, g.vy);
    R.az = axis_setup(ez, dz, L, g.nz, g.vz);
    R.smax = fminf(fminf(R.ax.last, R.ay.last), R.az.last);
    return R.smax < NR_FINF;  // false only when no axis is crossed at all
}

// Traces the ray (x0,y0,z0) -> (x1,y1,z1).  MODE 0: sum_j len_j * vol_j;
// MODE 1: in-volume chord length; MODE 2: full length |src - bin|; MODE 3:
// out[0] = the MODE 0 sum and out[1] = the chord, from one walk (the sum and
// sum_norm of rayTrace3D_GPU_direct_notexturememory, Tomo_OSTR.cu:327-610).
// Returns false when the ray misses the volume (the reference's status -1).
//
// MODE 0 walks in batches of K steps: the voxel indices and chord lengths of
// K segments are computed first (they do not depend on the volume), then the
// K gathers are issued together and accumulated in segment order, so a warp
// keeps K loads in flight instead of one.  The sum is bit-identical for every K.
template <int MODE, int K = 4>
__device__ __forceinline__ bool trace(const Geo& G, const float* __restrict__ vol, float x0,
                                      float y0, float z0, float x1, float y1, float z1,
                                      float* out) {
    const nr_geom& g = G.g;
    RayAxes R;
    if (!ray_axes<MODE == 2>(G, x0, y0, z0, x1, y1, z1, R)) return false;
    if (MODE == 2) {
        *out = R.L;  // Tomo_OSTR.cu:1172
        return true;
    }
    const Axis& ax = R.ax;
    const Axis& ay = R.ay;
    const Axis& az = R.az;
    const float smax = R.smax;
    if (MODE == 1) {
        *out = smax;
        return true;
    }
    if (MODE == 3) out[1] = smax;
    const int sx = ax.dir, sy = ay.dir * g.nx, sz = az.dir * g.nx * g.ny;
    int idx = (az.idx * g.ny + ay.idx) * g.nx + ax.idx;
    float tx = ax.first, ty = ay.first, tz = az.first;
    float cx = 0.f, cy = 0.f, cz = 0.f;
    float s = 0.f, sum = 0.f;
    while (s < smax) {
        float seg[K];
        int id[K];
        bool on[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            on[k] = s < smax;
            const float m = fmin3(tx, ty, tz);
            seg[k] = m - s;
            id[k] = idx;
            if (on[k]) {
                s = m;
                if (tx == m) {
                    cx += 1.f;
                    tx = __fmaf_rn(cx, ax.step, ax.first);
                    idx += sx;
                }
                if (ty == m) {
                    cy += 1.f;
                    ty = __fmaf_rn(cy, ay.step, ay.first);
                    idx += sy;
                }
                if (tz == m) {
                    cz += 1.f;
                    tz = __fmaf_rn(cz, az.step, az.first);
                    idx += sz;
                }
            }
        }
        float v[K];
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = on[k] ? __ldg(vol + id[k]) : 0.f;
#pragma unroll
        for (int k = 0; k < K; k++)
            if (on[k]) sum = __fmaf_rn(seg[k], v[k], sum);
    }
    *out = sum;
    return true;
}

}  // namespace nr
