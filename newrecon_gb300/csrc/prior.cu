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

// One sub-iteration's update, fused: SBP of h (subset views, [view][j][i]),
// the penalty, and the update_est step.  Writes x_out; flags non-finite values.
template <int POT>
__global__ void __launch_bounds__(128) update_kernel(
    const __grid_constant__ Geo G, const __grid_constant__ PriorW W,
    const float* __restrict__ x, float* __restrict__ x_out, const float* __restrict__ d,
    const float* __restrict__ h, const float* __restrict__ angles,
    const int32_t* __restrict__ index, int a0, int nv, float M, float beta, float delta,
    int* __restrict__ status) {
    __shared__ ViewSrc sv[UPD_VIEWS_SMEM];
    const nr_geom& g = G.g;
    for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < nv; t += blockDim.x * blockDim.y) {
        sv[t] = view_source(g, angles[index[a0 + t]]);
    }
    __syncthreads();
    const int ix = blockIdx.x * 32 + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    if (ix >= g.nx || iy >= g.ny) return;
    const int64_t v = ((int64_t)iz * g.ny + iy) * g.nx + ix;
    const float xc = x[v];
    // M * SBP(h)
    const float x1 = vox_x(g, ix), y1 = vox_y(g, iy), z1 = vox_z(g, iz);
    const int64_t B = (int64_t)g.nbx * g.nby;
    float capL = 0.f;
    for (int t = 0; t < nv; t++) {
        const ViewSrc vs = sv[t];
        const float ddx = vs.x0 - x1, ddy = vs.y0 - y1, ddz = vs.z0 - z1;
        const float dw = __fdiv_rn(vs.s2, ddx * ddx + ddy * ddy + ddz * ddz);
        if (z1 == vs.z0) continue;
        const float tt = __fdiv_rn(-g.detectorR - vs.z0, z1 - vs.z0);
        const float x2 = vs.x0 + (x1 - vs.x0) * tt;
        const float y2 = vs.y0 + (y1 - vs.y0) * tt;
        const float imb = __fdiv_rn(x2 - g.x_d0, g.bx);
        const float jmb = __fdiv_rn(y2 - g.y_d0, g.by);
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
    prior_sums<POT>(g, W, x, ix, iy, iz, xc, delta, 1.f / delta, &rdd, &rd);
    float xn = xc - __fdiv_rn(capL + beta * rd, d[v] + 2.f * beta * rdd);
    if (!(fabsf(xn) < __int_as_float(0x7f800000))) atomicOr(status, NR_FLAG_NONFINITE);
    x_out[v] = xn < 0.f ? 0.f : xn;
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
    dim3 blk(32, 4), grd(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz);
    update_kernel<POT><<<grd, blk, 0, st>>>(make_geo(g), make_weights(g.vz / g.vx), x, x_out, d, h,
                                            angles, index, a0, nv, M, beta, delta, status);
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
