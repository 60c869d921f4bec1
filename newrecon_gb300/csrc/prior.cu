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
#include "update.cuh"

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

// The SART prior gradient: prior += sum_k t/sqrt(1+(t/delta)^2) / dist_k with
// plain neighbour distances (G_Huber_prior, Tomo_OSTR.cu:258-325; W built
// with z ratio 1).  The RDD sums of prior_sums are dead here and drop out.
__global__ void __launch_bounds__(128) prior_grad_kernel(const __grid_constant__ Geo G,
                                                         const __grid_constant__ PriorW W,
                                                         float* __restrict__ prior,
                                                         const float* __restrict__ x,
                                                         float delta) {
    const nr_geom& g = G.g;
    const int ix = blockIdx.x * 32 + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    if (ix >= g.nx || iy >= g.ny) return;
    const int64_t v = ((int64_t)iz * g.ny + iy) * g.nx + ix;
    float rdd, rd;
    prior_sums<NR_POT_HYPERBOLA>(g, W, x, ix, iy, iz, x[v], delta, 1.f / delta, &rdd, &rd);
    prior[v] = prior[v] + rd;
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

// The separable back-projection tables of update.cuh for every view position
// a (subset order, angles[index[a]]), plane and column / row: grid (.., nz, A).
__global__ void __launch_bounds__(128) bp_table_kernel(const __grid_constant__ Geo G,
                                                       const float* __restrict__ angles,
                                                       const int32_t* __restrict__ index,
                                                       float4* __restrict__ tx,
                                                       float4* __restrict__ ty) {
    __shared__ ViewSrc src;
    const nr_geom& g = G.g;
    const int a = blockIdx.z, z = blockIdx.y;
    if (threadIdx.x == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    const float z1 = vox_z(g, z);
    const float tt = bp_tt(g, src, z1);
    const float inv_bx = 1.f / g.bx, inv_by = 1.f / g.by;
    const int64_t row = (int64_t)a * g.nz + z;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < g.nx + g.ny;
         q += gridDim.x * blockDim.x) {
        if (q < g.nx)
            tx[row * g.nx + q] = bp_entry_x(g, src, tt, q, inv_bx);
        else
            ty[row * g.ny + (q - g.nx)] = bp_entry_y(g, src, z1, tt, q - g.nx, inv_by);
    }
}

size_t bp_table_bytes(const nr_geom& g) {
    return (size_t)g.n_angles * g.nz * (g.nx + g.ny) * sizeof(float4);
}

nr_status launch_bp_tables(const nr_geom& g, const float* angles, const int32_t* index,
                           float4* tx, float4* ty, cudaStream_t st) {
    dim3 grd(cdiv((int64_t)g.nx + g.ny, 128), g.nz, g.n_angles);
    bp_table_kernel<<<grd, 128, 0, st>>>(make_geo(g), angles, index, tx, ty);
    return launch_status();
}

template <int POT, int ZC>
static nr_status launch_update_t(const nr_geom& g, int tile, const float* x, float* x_out, const float* d,
                                 const float* h, const float* angles, const int32_t* index,
                                 const BpTab& T, int a0, int nv, float M, float beta,
                                 float delta, int* status, const CUtensorMap* map,
                                 cudaStream_t st) {
    dim3 blk(UTX, UTY), grd(cdiv(g.nx, UTX), cdiv(g.ny, UTY), cdiv(g.nz, ZC));
    const Geo G = make_geo(g);
    const PriorW5 W = make_w5(g.vz / g.vx, delta);
    if (tile == NR_TILE_TMA && map) {
        if (nv == 1)
            update_tma_kernel<POT, ZC, 1><<<grd, blk, 0, st>>>(
                G, W, *map, x_out, d, h, angles, index, T, a0, nv, M, beta, delta, status);
        else
            update_tma_kernel<POT, ZC, 0><<<grd, blk, 0, st>>>(
                G, W, *map, x_out, d, h, angles, index, T, a0, nv, M, beta, delta, status);
    } else if (nv == 1 && tile == NR_TILE_2) {
        dim3 g2(cdiv(g.nx, U2X), cdiv(g.ny, UTY), cdiv(g.nz, ZC));
        update_x2_kernel<POT, ZC, 1><<<g2, blk, 0, st>>>(G, W, x, x_out, d, h, angles, index, T, a0,
                                                       nv, M, beta, delta, status);
    } else if (nv == 1)
        update_kernel<POT, ZC, 1><<<grd, blk, 0, st>>>(G, W, x, x_out, d, h, angles, index, T, a0,
                                                       nv, M, beta, delta, status);
    else
        update_kernel<POT, ZC, 0><<<grd, blk, 0, st>>>(G, W, x, x_out, d, h, angles, index, T, a0,
                                                       nv, M, beta, delta, status);
    return launch_status();
}

template <int POT>
static nr_status launch_update_z(const nr_geom& g, int zc, int tile, const float* x, float* x_out,
                                 const float* d, const float* h, const float* angles,
                                 const int32_t* index, const BpTab& T, int a0, int nv, float M,
                                 float beta, float delta, int* status, const CUtensorMap* map,
                                 cudaStream_t st) {
    switch (zc) {
    case 8:
        return launch_update_t<POT, 8>(g, tile, x, x_out, d, h, angles, index, T, a0, nv, M, beta, delta,
                                       status, map, st);
    case 32:
        return launch_update_t<POT, 32>(g, tile, x, x_out, d, h, angles, index, T, a0, nv, M, beta, delta,
                                        status, map, st);
    default:
        return launch_update_t<POT, 16>(g, tile, x, x_out, d, h, angles, index, T, a0, nv, M, beta, delta,
                                        status, map, st);
    }
}

nr_status launch_update(const nr_geom& g, int pot, int zc, int tile, const float* x, float* x_out,
                        const float* d, const float* h, const float* angles, const int32_t* index,
                        const BpTab& T, int a0, int nv, float M, float beta, float delta,
                        int* status, const CUtensorMap* map, cudaStream_t st) {
    if (nv > UPD_VIEWS_SMEM) return NR_ERR_BAD_ARGUMENT;
    switch (pot) {
    case NR_POT_Q2:
        return launch_update_z<NR_POT_Q2>(g, zc, tile, x, x_out, d, h, angles, index, T, a0, nv, M, beta,
                                          delta, status, map, st);
    case NR_POT_LANGE:
        return launch_update_z<NR_POT_LANGE>(g, zc, tile, x, x_out, d, h, angles, index, T, a0, nv, M, beta,
                                             delta, status, map, st);
    case NR_POT_HYPERBOLA:
        return launch_update_z<NR_POT_HYPERBOLA>(g, zc, tile, x, x_out, d, h, angles, index, T, a0, nv, M,
                                                 beta, delta, status, map, st);
    case NR_POT_HUBER:
        return launch_update_z<NR_POT_HUBER>(g, zc, tile, x, x_out, d, h, angles, index, T, a0, nv, M, beta,
                                             delta, status, map, st);
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

NR_API nr_status nr_prior_sart(const nr_geom* g, float* prior, const float* x, float delta,
                               void* stream) {
    if (!geom_ok(g)) return NR_ERR_BAD_GEOMETRY;
    if (!prior || !x || prior == x) return NR_ERR_BAD_ARGUMENT;
    if (delta == 0.f || !(delta == delta)) return NR_ERR_BAD_ARGUMENT;  // Tomo_OSTR.cu:2260-2263
    if (g->nz > 65535) return NR_ERR_BAD_GEOMETRY;
    dim3 blk(32, 4), grd(cdiv(g->nx, 32), cdiv(g->ny, 4), g->nz);
    prior_grad_kernel<<<grd, blk, 0, as_stream(stream)>>>(make_geo(*g), make_weights(1.f), prior,
                                                          x, delta);
    return launch_status();
}
