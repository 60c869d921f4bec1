// bp.cu -- voxel-driven bilinear back projector (SBP), a deterministic gather.
//
// One thread per voxel, threads along x.  For every view of the range the
// voxel centre is projected from the source onto the detector plane, the
// detector is bilinearly interpolated with the reference's edge rules, the
// sample is weighted by Vsize_z * depth_weight and the per-view terms are
// summed in view order; the voxel's accumulator gets one add.  No atomics,
// so results are bit-reproducible run to run.  Restates the arithmetic of
// backprj_gpu_manyviews_SBP, Tomo_OSTR.cu:1553-1734.
//
// Along a warp (32 consecutive x voxels of one (y, z) row) the projected
// detector row j and weight fracJ are the same for every lane and the columns
// i are consecutive, so with the [j][i] detector layout the four taps of a
// warp fall on 2 detector rows x ~33 consecutive floats: coalesced.
#include "common.cuh"

namespace nr {

constexpr int BP_VIEWS_SMEM = 64;

__device__ __forceinline__ void load_views(const nr_geom& g, ViewSrc* sv,
                                           const float* __restrict__ angles,
                                           const int32_t* __restrict__ index, int a0, int nv) {
    for (int t = threadIdx.x; t < nv; t += blockDim.x) {
        const int s = index ? index[a0 + t] : a0 + t;
        sv[t] = view_source(g, angles[s]);
    }
}

// One view's SBP term for voxel centre (x1,y1,z1) reading view plane p.
// SENS also returns in *sens the same interpolation of a detector of ones
// (the OS-SART sensitivity, Tomo_OSTR.cu:1838-1882).
template <bool JI, bool SENS = false>
__device__ __forceinline__ float sbp_term(const nr_geom& g, const ViewSrc& v, float x1, float y1,
                                          float z1, const float* __restrict__ p,
                                          float* sens = nullptr) {
    const float ddx = v.x0 - x1, ddy = v.y0 - y1, ddz = v.z0 - z1;
    const float depth_weight = __fdiv_rn(v.s2, ddx * ddx + ddy * ddy + ddz * ddz);  // :1634
    if (SENS) *sens = 0.f;
    if (z1 == v.z0) return 0.f;
    const float t = __fdiv_rn(-g.detectorR - v.z0, z1 - v.z0);
    const float x2 = v.x0 + (x1 - v.x0) * t;
    const float y2 = v.y0 + (y1 - v.y0) * t;
    const float imb = __fdiv_rn(x2 - g.x_d0, g.bx);
    const float jmb = __fdiv_rn(y2 - g.y_d0, g.by);
    int ilb = (int)floorf(imb);
    if (imb < (float)ilb + 0.5f) ilb -= 1;
    int jlb = (int)floorf(jmb);
    if (jmb < (float)jlb + 0.5f) jlb -= 1;
    const float fracI = imb - ((float)ilb + 0.5f);
    const float fracJ = jmb - ((float)jlb + 0.5f);
    const int NBX = g.nbx, NBY = g.nby;
    auto at = [&](int i, int j) -> float {
        return __ldg(p + (JI ? (int64_t)j * NBX + i : (int64_t)i * NBY + j));
    };
    // Tap rules of Tomo_OSTR.cu:1684-1715: each tap contributes only when it
    // lies on the detector; no renormalisation.
    float d1 = 0.f, d2 = 0.f, s1 = 0.f, s2 = 0.f;
    const bool i0 = (ilb < NBX) && (ilb >= 0);
    const bool i1 = (ilb < NBX - 1) && (ilb >= -1);
    const bool j0 = (jlb < NBY) && (jlb >= 0);
    const bool j1 = (jlb < NBY - 1) && (jlb >= -1);
    if (i0 && j0) {
        d1 = (1.f - fracI) * at(ilb, jlb);
        s1 = 1.f - fracI;
    }
    if (i1 && j0) {
        d1 = d1 + fracI * at(ilb + 1, jlb);
        s1 = s1 + fracI;
    }
    if (i0 && j1) {
        d2 = (1.f - fracI) * at(ilb, jlb + 1);
        s2 = 1.f - fracI;
    }
    if (i1 && j1) {
        d2 = d2 + fracI * at(ilb + 1, jlb + 1);
        s2 = s2 + fracI;
    }
    const float u = (1.f - fracJ) * d1 + fracJ * d2;
    if (SENS) *sens = ((1.f - fracJ) * s1 + fracJ * s2) * g.vz * depth_weight;
    return u * g.vz * depth_weight;
}

// vol[v] += sum_{views} SBP term.  prj planes are consecutive per view
// (view a-a0 at prj + (a-a0)*B).  index == nullptr means identity order.
template <bool JI>
__global__ void __launch_bounds__(128) bp_kernel(const __grid_constant__ Geo G,
                                                 float* __restrict__ vol,
                                                 const float* __restrict__ prj,
                                                 const float* __restrict__ angles,
                                                 const int32_t* __restrict__ index, int a0,
                                                 int nv) {
    __shared__ ViewSrc sv[BP_VIEWS_SMEM];
    const nr_geom& g = G.g;
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y, iz = blockIdx.z;
    const float x1 = vox_x(g, ix), y1 = vox_y(g, iy), z1 = vox_z(g, iz);
    const int64_t B = (int64_t)g.nbx * g.nby;
    float total = 0.f;
    for (int c0 = 0; c0 < nv; c0 += BP_VIEWS_SMEM) {
        const int cn = min(BP_VIEWS_SMEM, nv - c0);
        __syncthreads();
        load_views(g, sv, angles, index, a0 + c0, cn);
        __syncthreads();
        if (ix < g.nx)
            for (int t = 0; t < cn; t++)
                total = total + sbp_term<JI>(g, sv[t], x1, y1, z1, prj + (int64_t)(c0 + t) * B);
    }
    if (ix < g.nx) {
        const int64_t v = ((int64_t)iz * g.ny + iy) * g.nx + ix;
        vol[v] = vol[v] + total;
    }
}

// OS-SART update in place over views [a0, a0+nv) of the [view][i][j]
// difference: x += lambda (sum_u + beta prior) / sum_sens (both terms 0 where
// sum_sens = 0), then x = max(x, 0).  prior == nullptr is
// backprj_OSSART_gpu_manyviews (Tomo_OSTR.cu:1737-1936), otherwise
// backprj_OSSART_R_gpu_manyviews (:1938-2143).  Each voxel reads and writes
// only itself, so the update is safe in place.
__global__ void __launch_bounds__(128) bp_ossart_kernel(const __grid_constant__ Geo G,
                                                        float* __restrict__ vol,
                                                        const float* __restrict__ prj,
                                                        const float* __restrict__ prior,
                                                        const float* __restrict__ angles,
                                                        const int32_t* __restrict__ index,
                                                        int a0, int nv, float lambda, float beta) {
    __shared__ ViewSrc sv[BP_VIEWS_SMEM];
    const nr_geom& g = G.g;
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y, iz = blockIdx.z;
    const float x1 = vox_x(g, ix), y1 = vox_y(g, iy), z1 = vox_z(g, iz);
    const int64_t B = (int64_t)g.nbx * g.nby;
    float total = 0.f, total_sens = 0.f;
    for (int c0 = 0; c0 < nv; c0 += BP_VIEWS_SMEM) {
        const int cn = min(BP_VIEWS_SMEM, nv - c0);
        __syncthreads();
        load_views(g, sv, angles, index, a0 + c0, cn);
        __syncthreads();
        if (ix < g.nx)
            for (int t = 0; t < cn; t++) {
                float sn;
                total = total + sbp_term<false, true>(g, sv[t], x1, y1, z1,
                                                      prj + (int64_t)(c0 + t) * B, &sn);
                total_sens = total_sens + sn;
            }
    }
    if (ix < g.nx) {
        const int64_t v = ((int64_t)iz * g.ny + iy) * g.nx + ix;
        float u = 0.f, bt = 0.f;
        if (total_sens != 0.f) {
            u = __fdiv_rn(total, total_sens);
            if (prior) bt = __fdiv_rn(beta * prior[v], total_sens);
        }
        const float xn = vol[v] + lambda * (u + bt);
        vol[v] = xn < 0.f ? 0.f : xn;
    }
}

nr_status launch_bp(const nr_geom& g, bool ji, float* vol, const float* prj, const float* angles,
                    const int32_t* index, int a0, int nv, cudaStream_t st) {
    dim3 blk(128), grd(cdiv(g.nx, 128), g.ny, g.nz);
    if (ji)
        bp_kernel<true><<<grd, blk, 0, st>>>(make_geo(g), vol, prj, angles, index, a0, nv);
    else
        bp_kernel<false><<<grd, blk, 0, st>>>(make_geo(g), vol, prj, angles, index, a0, nv);
    return launch_status();
}

}  // namespace nr

using namespace nr;

NR_API nr_status nr_bp_sbp(const nr_geom* g, float* vol, const float* prj, const int32_t* index,
                           const float* angles, int32_t a0, int32_t a1, void* stream) {
    if (!geom_ok(g)) return NR_ERR_BAD_GEOMETRY;
    if (!vol || !prj || !index || !angles || a0 < 0 || a1 < a0) return NR_ERR_BAD_ARGUMENT;
    if (g->ny > 65535 || g->nz > 65535) return NR_ERR_BAD_GEOMETRY;
    if (a1 == a0) return NR_OK;
    return launch_bp(*g, false, vol, prj, angles, index, a0, a1 - a0, as_stream(stream));
}

NR_API nr_status nr_bp_ossart(const nr_geom* g, float* x, const float* diff, const float* prior,
                              const int32_t* index, const float* angles, int32_t a0, int32_t a1,
                              float lambda, float beta, void* stream) {
    if (!geom_ok(g)) return NR_ERR_BAD_GEOMETRY;
    if (!x || !diff || !index || !angles || a0 < 0 || a1 < a0) return NR_ERR_BAD_ARGUMENT;
    if (prior == x) return NR_ERR_BAD_ARGUMENT;
    if (g->ny > 65535 || g->nz > 65535) return NR_ERR_BAD_GEOMETRY;
    if (a1 == a0) return NR_OK;
    dim3 blk(128), grd(cdiv(g->nx, 128), g->ny, g->nz);
    bp_ossart_kernel<<<grd, blk, 0, as_stream(stream)>>>(make_geo(*g), x, diff, prior, angles,
                                                         index, a0, a1 - a0, lambda, beta);
    return launch_status();
}
