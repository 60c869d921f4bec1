// prior.cu -- 26-neighbour edge-preserving penalty and the fused OSTR update.
//
// For voxel j and each of its 26 neighbours k (t = x_j - x_k, neighbour
// weight w = 1/sqrt(dx^2 + dy^2 + (dz * z_xy_ratio)^2)):
//     RDD_j += w * omega(t),   RD_j += w * omega(t) * t
// with omega = 1 (Q2), 1/(1+|t|/delta) (Lange), 1/sqrt(1+(t/delta)^2)
// (hyperbola) or min(1, delta/|t|) (Huber).  A neighbour outside the volume
// is replaced by the voxel itself: t = 0, omega = 1, so its weight still adds
// to RDD (Tomo_OSTR.cu:118-255).
//
// The fused kernel computes, per voxel and in one pass,
//     capL = M * SBP(h over the subset views)          (Tomo_OSTR_gold.cpp:759-771)
//     RDD, RD as above from the current x              (:775)
//     x' = max(0, x - (capL + beta RD) / (d + 2 beta RDD))   (update_est :265-295)
// and writes x' to a second buffer (neighbours must see the old x).
#include <cmath>
#include <utility>

#include "common.cuh"

namespace nr {

nr_status launch_bp(const nr_geom& g, bool ji, float* vol, const float* prj, const float* angles,
                    const int32_t* index, int a0, int nv, cudaStream_t st);

struct PriorW {
    float w[27];  // weight of neighbour (dx,dy,dz) at ((dz+1)*3+(dy+1))*3+(dx+1); centre 0
};

__host__ inline PriorW make_weights(float zxy) {
    PriorW p;
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                // distance as the reference forms it: float sqrt of a float sum,
                // then 1.0/distance in double, rounded once (Tomo_OSTR.cu:229).
                float dist = std::sqrt((float)(dx * dx + dy * dy) + (float)(dz * dz) * zxy * zxy);
                int k = ((dz + 1) * 3 + (dy + 1)) * 3 + (dx + 1);
                p.w[k] = (dist == 0.f) ? 0.f : (float)(1.0 / (double)dist);
            }
    return p;
}

// omega(t) with inv_delta = 1/delta.
template <int POT>
__device__ __forceinline__ float omega(float t, float delta, float inv_delta) {
    if (POT == NR_POT_Q2) return 1.f;
    if (POT == NR_POT_LANGE) return __fdividef(1.f, __fmaf_rn(fabsf(t), inv_delta, 1.f));
    if (POT == NR_POT_HYPERBOLA) {
        const float u = t * inv_delta;
        return rsqrtf(__fmaf_rn(u, u, 1.f));
    }
    const float a = fabsf(t);  // Huber
    return a <= delta ? 1.f : __fdividef(delta, a);
}

// RDD/RD sums over the 26 neighbours of (ix, iy, iz), read through L1.
template <int POT>
__device__ __forceinline__ void prior_sums(const nr_geom& g, const PriorW& W,
                                           const float* __restrict__ x, int ix, int iy, int iz,
                                           float xc, float delta, float inv_delta, float* rdd,
                                           float* rd) {
    float sdd = 0.f, sd = 0.f;
    const int64_t plane = (int64_t)g.nx * g.ny;
#pragma unroll
    for (int dz = -1; dz <= 1; dz++) {
#pragma unroll
        for (int dy = -1; dy <= 1; dy++) {
#pragma unroll
            for (int dx = -1; dx <= 1; dx++) {
                if (dx == 0 && dy == 0 && dz == 0) continue;
                const int kx = ix + dx, ky = iy + dy, kz = iz + dz;
                const bool in = (unsigned)kx < (unsigned)g.nx && (unsigned)ky < (unsigned)g.ny &&
                                (unsigned)kz < (unsigned)g.nz;
                float t = 0.f;
                if (in) t = xc - __ldg(x + (int64_t)kz * plane + (int64_t)ky * g.nx + kx);
                const float wo = W.w[((dz + 1) * 3 + (dy + 1)) * 3 + (dx + 1)] *
                                 omega<POT>(t, delta, inv_delta);
                sdd += wo;
                sd = __fmaf_rn(wo, t, sd);
            }
        }
    }
    *rdd = sdd;
    *rd = sd;
}

// Reference-shaped prior: RDD += ..., RD += ... (prior_GPU_OSTR / _Q2).
template <int POT>
__global__ void __launch_bounds__(128) prior_kernel(const __grid_constant__ Geo G,
                                                    const __grid_constant__ PriorW W,
                                                    float* __restrict__ RDD,
                                                    float* __restrict__ RD,
                                                    const float* __restrict__ x, float delta) {
    const nr_geom& g = G.g;
    const int ix = blockIdx.x * 32 + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    if (ix >= g.nx || iy >= g.ny) return;
    const int64_t v = ((int64_t)iz * g.ny + iy) * g.nx + ix;
    float rdd, rd;
    prior_sums<POT>(g, W, x, ix, iy, iz, x[v], delta, 1.f / delta, &rdd, &rd);
    RDD[v] = RDD[v] + rdd;
    RD[v] = RD[v] + rd;
}

constexpr int UPD_VIEWS_SMEM = 32;
constexpr int UTX = 32, UTY = 8, UZC = 16;      // tile: 32 x 8 columns, 16 planes per block
constexpr int USW = UTX + 2, USH = UTY + 2;     // plane tile with a 1-voxel halo
constexpr int UPLANE = USW * USH;

// The five distinct neighbour weights 1/sqrt(dx^2+dy^2+(dz zr)^2) of the
// 26-neighbourhood (in-plane face, in-plane diagonal, z face, z edge, z
// corner) and the same times delta (Huber).
struct PriorW5 {
    float w1, w2, wz, wz1, wz2;
    float d1, d2, dz, dz1, dz2;
};

__host__ inline PriorW5 make_w5(float zxy, float delta) {
    auto w = [&](int dx, int dy, int dz) {
        const float dist = std::sqrt((float)(dx * dx + dy * dy) + (float)(dz * dz) * zxy * zxy);
        return (float)(1.0 / (double)dist);
    };
    PriorW5 p;
    p.w1 = w(1, 0, 0);
    p.w2 = w(1, 1, 0);
    p.wz = w(0, 0, 1);
    p.wz1 = w(1, 0, 1);
    p.wz2 = w(1, 1, 1);
    p.d1 = p.w1 * delta;
    p.d2 = p.w2 * delta;
    p.dz = p.wz * delta;
    p.dz1 = p.wz1 * delta;
    p.dz2 = p.wz2 * delta;
    return p;
}

// Approximate reciprocal / reciprocal square root (the MUFU unit, <= 1 ulp
// relative error; arguments here are >= 1 or >= delta, never denormal).
__device__ __forceinline__ float rcp_approx(float v) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float v) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}

// Neighbour K = ((dz+1)*3 + (dy+1))*3 + (dx+1) of the centre at offset
// `base` in the shared-memory planes: adds w omega(t) to sdd and w omega(t) t
// to sd (two accumulator pairs, even/odd K, to shorten the dependency
// chains).  EDGE: out-of-volume cells hold NaN and count as t = 0.
template <int POT, bool EDGE, int K>
__device__ __forceinline__ void nb_term(const float* __restrict__ pb, const float* __restrict__ pc,
                                        const float* __restrict__ pa, int base, float xc,
                                        const PriorW5& W, float delta, float inv_delta,
                                        float& sdd0, float& sd0, float& sdd1, float& sd1) {
    constexpr int dz = K / 9 - 1, dy = (K / 3) % 3 - 1, dx = K % 3 - 1;
    if constexpr (K == 13) {
        return;  // the centre itself
    } else {
        constexpr int nxy = (dx != 0) + (dy != 0);
        const float* pl = dz < 0 ? pb : (dz == 0 ? pc : pa);
        float t = xc - pl[base + dy * USW + dx];
        if (EDGE) t = (t == t) ? t : 0.f;
        float w, wd;
        if (dz == 0) {
            w = nxy == 1 ? W.w1 : W.w2;
            wd = nxy == 1 ? W.d1 : W.d2;
        } else {
            w = nxy == 0 ? W.wz : (nxy == 1 ? W.wz1 : W.wz2);
            wd = nxy == 0 ? W.dz : (nxy == 1 ? W.dz1 : W.dz2);
        }
        float wo;
        if (POT == NR_POT_Q2) {
            wo = w;
        } else if (POT == NR_POT_LANGE) {
            wo = w * rcp_approx(__fmaf_rn(fabsf(t), inv_delta, 1.f));
        } else if (POT == NR_POT_HYPERBOLA) {
            const float u = t * inv_delta;
            wo = w * rsqrt_approx(__fmaf_rn(u, u, 1.f));
        } else {
            wo = wd * rcp_approx(fmaxf(fabsf(t), delta));  // w min(1, delta/|t|)
        }
        if (K & 1) {
            sdd1 += wo;
            sd1 = __fmaf_rn(wo, t, sd1);
        } else {
            sdd0 += wo;
            sd0 = __fmaf_rn(wo, t, sd0);
        }
    }
}

template <int POT, bool EDGE, int... Ks>
__device__ __forceinline__ void prior_all(std::integer_sequence<int, Ks...>,
                                          const float* __restrict__ pb,
                                          const float* __restrict__ pc,
                                          const float* __restrict__ pa, int base, float xc,
                                          const PriorW5& W, float delta, float inv_delta,
                                          float* rdd, float* rd) {
    float a0 = 0.f, b0 = 0.f, a1 = 0.f, b1 = 0.f;
    (nb_term<POT, EDGE, Ks>(pb, pc, pa, base, xc, W, delta, inv_delta, a0, b0, a1, b1), ...);
    *rdd = a0 + a1;
    *rd = b0 + b1;
}

// One sub-iteration's update, fused: SBP of h (subset views, [view][j][i]),
// the penalty, and the update_est step.  Each block owns a 32 x 8 tile of
// (x, y) columns and walks UZC planes in z, keeping planes z-1, z, z+1 of x
// (with halo) in a 3-slot shared-memory ring, so every neighbour read is a
// shared-memory load at a fixed offset.  The global loads of plane z+2 are
// issued before plane z is computed (register prefetch), so they overlap the
// arithmetic.  Writes x_out; flags non-finite values.
template <int POT>
__global__ void __launch_bounds__(256) update_kernel(
    const __grid_constant__ Geo G, const __grid_constant__ PriorW5 W,
    const float* __restrict__ x, float* __restrict__ x_out, const float* __restrict__ d,
    const float* __restrict__ h, const float* __restrict__ angles,
    const int32_t* __restrict__ index, int a0, int nv, float M, float beta, float delta,
    int* __restrict__ status) {
    __shared__ float tile[3][UPLANE];
    __shared__ ViewSrc sv[UPD_VIEWS_SMEM];
    const nr_geom& g = G.g;
    const int tid = threadIdx.y * UTX + threadIdx.x;
    for (int t = tid; t < nv; t += UTX * UTY) sv[t] = view_source(g, angles[index[a0 + t]]);
    const int x0t = blockIdx.x * UTX, y0t = blockIdx.y * UTY;
    const int zb = blockIdx.z * UZC, ze = min(zb + UZC, g.nz);
    const int64_t plane = (int64_t)g.nx * g.ny;
    // This thread's (at most two) cells of a halo plane tile.
    constexpr int NT = UTX * UTY;
    static_assert(UPLANE <= 2 * NT, "two cells per thread");
    const int e1 = tid + NT;
    const bool has1 = e1 < UPLANE;
    auto cell_off = [&](int k, bool& ok) -> int64_t {
        const int r = k / USW, c = k - r * USW;
        const int gx = x0t - 1 + c, gy = y0t - 1 + r;
        ok = gx >= 0 && gx < g.nx && gy >= 0 && gy < g.ny;
        return ok ? (int64_t)gy * g.nx + gx : 0;
    };
    bool ok0, ok1 = false;
    const int64_t off0 = cell_off(tid, ok0);
    const int64_t off1 = has1 ? cell_off(e1, ok1) : 0;
    const float qnan = __int_as_float(0x7fc00000);  // outside the volume
    auto fetch = [&](int z, float& v0, float& v1) {
        const bool zin = z >= 0 && z < g.nz;
        v0 = (zin && ok0) ? __ldg(x + (int64_t)z * plane + off0) : qnan;
        v1 = (zin && ok1) ? __ldg(x + (int64_t)z * plane + off1) : qnan;
    };
    float* pb = tile[0];
    float* pc = tile[1];
    float* pa = tile[2];
    {
        float v0, v1;
        fetch(zb - 1, v0, v1);
        pb[tid] = v0;
        if (has1) pb[e1] = v1;
        fetch(zb, v0, v1);
        pc[tid] = v0;
        if (has1) pc[e1] = v1;
    }
    float n0, n1;
    fetch(zb + 1, n0, n1);
    const int ix = x0t + threadIdx.x, iy = y0t + threadIdx.y;
    const bool active = ix < g.nx && iy < g.ny;
    const bool edge_xy = x0t == 0 || x0t + UTX >= g.nx || y0t == 0 || y0t + UTY >= g.ny;
    const float inv_delta = 1.f / delta;
    const float inv_bx = 1.f / g.bx, inv_by = 1.f / g.by;
    const float x1 = vox_x(g, ix), y1 = vox_y(g, iy);
    const int64_t B = (int64_t)g.nbx * g.nby;
    const int r = threadIdx.y + 1, c = threadIdx.x + 1;
    for (int z = zb; z < ze; z++) {
        pa[tid] = n0;
        if (has1) pa[e1] = n1;
        __syncthreads();
        if (z + 1 < ze) fetch(z + 2, n0, n1);
        if (active) {
            const int64_t v = (int64_t)z * plane + (int64_t)iy * g.nx + ix;
            const float dv = __ldg(d + v);
            const float xc = pc[r * USW + c];
            const float z1 = vox_z(g, z);
            // M * SBP(h): the arithmetic of bp.cu's sbp_term on the [j][i]
            // layout, with reciprocal multiplies in place of divisions.
            float capL = 0.f;
            for (int t = 0; t < nv; t++) {
                const ViewSrc vs = sv[t];
                const float ddx = vs.x0 - x1, ddy = vs.y0 - y1, ddz = vs.z0 - z1;
                const float dw = __fdividef(vs.s2, ddx * ddx + ddy * ddy + ddz * ddz);
                if (z1 == vs.z0) continue;
                const float tt = __fdividef(-g.detectorR - vs.z0, z1 - vs.z0);
                const float x2 = vs.x0 + (x1 - vs.x0) * tt;
                const float y2 = vs.y0 + (y1 - vs.y0) * tt;
                const float imb = (x2 - g.x_d0) * inv_bx;
                const float jmb = (y2 - g.y_d0) * inv_by;
                int ilb = (int)floorf(imb);
                if (imb < (float)ilb + 0.5f) ilb -= 1;
                int jlb = (int)floorf(jmb);
                if (jmb < (float)jlb + 0.5f) jlb -= 1;
                const float fracI = imb - ((float)ilb + 0.5f);
                const float fracJ = jmb - ((float)jlb + 0.5f);
                const float* p = h + (int64_t)t * B;
                const bool i0 = (ilb < g.nbx) && (ilb >= 0);
                const bool i1 = (ilb < g.nbx - 1) && (ilb >= -1);
                const bool j0 = (jlb < g.nby) && (jlb >= 0);
                const bool j1 = (jlb < g.nby - 1) && (jlb >= -1);
                float d1 = 0.f, d2 = 0.f;
                const int64_t r0 = (int64_t)jlb * g.nbx, r1 = r0 + g.nbx;
                if (i0 && j0) d1 = (1.f - fracI) * __ldg(p + r0 + ilb);
                if (i1 && j0) d1 = d1 + fracI * __ldg(p + r0 + ilb + 1);
                if (i0 && j1) d2 = (1.f - fracI) * __ldg(p + r1 + ilb);
                if (i1 && j1) d2 = d2 + fracI * __ldg(p + r1 + ilb + 1);
                capL = capL + ((1.f - fracJ) * d1 + fracJ * d2) * g.vz * dw;
            }
            capL = M * capL;
            float rdd, rd;
            const int base = r * USW + c;
            if (edge_xy || z == 0 || z == g.nz - 1)
                prior_all<POT, true>(std::make_integer_sequence<int, 27>{}, pb, pc, pa, base, xc, W,
                                     delta, inv_delta, &rdd, &rd);
            else
                prior_all<POT, false>(std::make_integer_sequence<int, 27>{}, pb, pc, pa, base, xc, W,
                                      delta, inv_delta, &rdd, &rd);
            const float xn = xc - __fdividef(capL + beta * rd, dv + 2.f * beta * rdd);
            if (!(fabsf(xn) < __int_as_float(0x7f800000))) atomicOr(status, NR_FLAG_NONFINITE);
            x_out[v] = xn < 0.f ? 0.f : xn;
        }
        __syncthreads();
        float* t = pb;
        pb = pc;
        pc = pa;
        pa = t;
    }
}

template <int POT>
static nr_status launch_prior_t(const nr_geom& g, float* RDD, float* RD, const float* x,
                                float delta, float zxy, cudaStream_t st) {
    dim3 blk(32, 4), grd(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz);
    prior_kernel<POT><<<grd, blk, 0, st>>>(make_geo(g), make_weights(zxy), RDD, RD, x, delta);
    return launch_status();
}

nr_status launch_prior(const nr_geom& g, int pot, float* RDD, float* RD, const float* x,
                       float delta, float zxy, cudaStream_t st) {
    switch (pot) {
    case NR_POT_Q2: return launch_prior_t<NR_POT_Q2>(g, RDD, RD, x, delta, zxy, st);
    case NR_POT_LANGE: return launch_prior_t<NR_POT_LANGE>(g, RDD, RD, x, delta, zxy, st);
    case NR_POT_HYPERBOLA: return launch_prior_t<NR_POT_HYPERBOLA>(g, RDD, RD, x, delta, zxy, st);
    case NR_POT_HUBER: return launch_prior_t<NR_POT_HUBER>(g, RDD, RD, x, delta, zxy, st);
    default: return NR_ERR_BAD_ARGUMENT;
    }
}

template <int POT>
static nr_status launch_update_t(const nr_geom& g, const float* x, float* x_out, const float* d,
                                 const float* h, const float* angles, const int32_t* index,
                                 int a0, int nv, float M, float beta, float delta, int* status,
                                 cudaStream_t st) {
    dim3 blk(UTX, UTY), grd(cdiv(g.nx, UTX), cdiv(g.ny, UTY), cdiv(g.nz, UZC));
    update_kernel<POT><<<grd, blk, 0, st>>>(make_geo(g), make_w5(g.vz / g.vx, delta), x,
                                            x_out, d, h, angles, index, a0, nv, M, beta, delta,
                                            status);
    return launch_status();
}

nr_status launch_update(const nr_geom& g, int pot, const float* x, float* x_out, const float* d,
                        const float* h, const float* angles, const int32_t* index, int a0, int nv,
                        float M, float beta, float delta, int* status, cudaStream_t st) {
    if (nv > UPD_VIEWS_SMEM) return NR_ERR_BAD_ARGUMENT;
    switch (pot) {
    case NR_POT_Q2:
        return launch_update_t<NR_POT_Q2>(g, x, x_out, d, h, angles, index, a0, nv, M, beta, delta,
                                          status, st);
    case NR_POT_LANGE:
        return launch_update_t<NR_POT_LANGE>(g, x, x_out, d, h, angles, index, a0, nv, M, beta,
                                             delta, status, st);
    case NR_POT_HYPERBOLA:
        return launch_update_t<NR_POT_HYPERBOLA>(g, x, x_out, d, h, angles, index, a0, nv, M, beta,
                                                 delta, status, st);
    case NR_POT_HUBER:
        return launch_update_t<NR_POT_HUBER>(g, x, x_out, d, h, angles, index, a0, nv, M, beta,
                                             delta, status, st);
    default: return NR_ERR_BAD_ARGUMENT;
    }
}

}  // namespace nr

using namespace nr;

NR_API nr_status nr_prior(const nr_geom* g, float* RDD, float* RD, const float* x,
                          int32_t potential, float delta, float z_xy_ratio, void* stream) {
    if (!geom_ok(g)) return NR_ERR_BAD_GEOMETRY;
    if (!RDD || !RD || !x) return NR_ERR_BAD_ARGUMENT;
    if (potential != NR_POT_Q2 && !(delta > 0.f)) return NR_ERR_BAD_ARGUMENT;  // Tomo_OSTR.cu:2232
    if (g->nz > 65535) return NR_ERR_BAD_GEOMETRY;
    return launch_prior(*g, potential, RDD, RD, x, potential == NR_POT_Q2 ? 1.f : delta,
                        z_xy_ratio, as_stream(stream));
}
