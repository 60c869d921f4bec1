// fp.cu -- ray-driven cone-beam forward projectors (Siddon exact chord lengths).
//
// One thread per detector bin, a warp per 32 consecutive bins of one detector
// column j (lanes along i, the detector x axis).  Adjacent lanes trace nearly
// parallel rays 1 bin apart in x, so at every step their volume reads fall on
// the same few 128-byte lines of one volume row (the volume is x-fastest):
// the gathers coalesce.  Views of a launch run on gridDim.z.  The walk itself
// is in siddon.cuh.
#include <cudaTypedefs.h>

#include "project.cuh"
#include "slab.cuh"

namespace nr {

// Reference-shaped projector: out[(a-a0)] = cos * line integral (MODE 0) or
// gamma (MODE 1 chord, MODE 2 length); missed rays leave out untouched
// (Tomo_OSTR.cu:1367-1373, :1440-1446).
template <int MODE, bool JI>
__global__ void __launch_bounds__(128) fp_kernel(const __grid_constant__ Geo G,
                                                 const float* __restrict__ vol,
                                                 float* __restrict__ out,
                                                 const float* __restrict__ angles,
                                                 const int32_t* __restrict__ index, int a0) {
    __shared__ ViewSrc src;
    const nr_geom& g = G.g;
    const int a = a0 + blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nbx || j >= g.nby) return;
    float v;
    if (trace<MODE>(G, vol, src.x0, src.y0, src.z0, bin_x(g, i), bin_y(g, j), -g.detectorR, &v)) {
        const int64_t o = (int64_t)blockIdx.z * g.nbx * g.nby + bin_off<JI>(g, i, j);
        out[o] = (MODE == 0) ? v * src.ct : v;
    }
}

// SART projector: est = line integral (times cos theta when COS) and norm =
// in-volume chord of the same walk; missed rays leave both untouched
// (ray_trace_gpu_manyangles_direct_notexturememory{,_cos},
// Tomo_OSTR.cu:1177-1311).
template <bool COS>
__global__ void __launch_bounds__(128) fp_sart_kernel(const __grid_constant__ Geo G,
                                                      const float* __restrict__ vol,
                                                      float* __restrict__ est,
                                                      float* __restrict__ norm,
                                                      const float* __restrict__ angles,
                                                      const int32_t* __restrict__ index, int a0) {
    __shared__ ViewSrc src;
    const nr_geom& g = G.g;
    const int a = a0 + blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nbx || j >= g.nby) return;
    float v[2];
    if (trace<3>(G, vol, src.x0, src.y0, src.z0, bin_x(g, i), bin_y(g, j), -g.detectorR, v)) {
        const int64_t o = (int64_t)blockIdx.z * g.nbx * g.nby + bin_off<false>(g, i, j);
        est[o] = COS ? v[0] * src.ct : v[0];
        norm[o] = v[1];
    }
}

// 2 x 2 super-sampled projection: the fixed fprojectCB1_4R_GPU_SART
// (Tomo_OSTR.cu:1453-1550, 2398-2433).  One thread per sub-ray: sub-bin
// (is, js) of the 2 BINSx x 2 BINSy sub-detector, centre
// x_d0 + (is + 0.5) Bsize_x / 2 (:1491-1492); a block is 32 x 8 sub-rays =
// 16 x 4 bins of one view.  Bin (i, j) gets (((s00 + s10) + s01) + s11) / 4,
// s_ab the sub-ray (2i+a, 2j+b) with missed sub-rays 0 -- the merge of
// :1517-1550 as intended (there the fourth index is never assigned and the
// sub-ray buffer is read as the caller left it) -- times cos theta when COS.
// out: JI ? [view][j][i] (the reference merge's layout) : [view][i][j].
// sub, when given: [view][2 BINSy][2 BINSx] sub-ray sums (missed untouched).
template <bool COS, bool JI>
__global__ void __launch_bounds__(256) fp_4r_kernel(const __grid_constant__ Geo G,
                                                    const float* __restrict__ vol,
                                                    float* __restrict__ out,
                                                    float* __restrict__ sub,
                                                    const float* __restrict__ angles,
                                                    const int32_t* __restrict__ index, int a0) {
    __shared__ ViewSrc src;
    __shared__ float tile[8][33];
    const nr_geom& g = G.g;
    const int a = a0 + blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int is = blockIdx.x * 32 + tx, js = blockIdx.y * 8 + ty;
    const int nbx2 = 2 * g.nbx, nby2 = 2 * g.nby;
    const bool on = is < nbx2 && js < nby2;
    float v = 0.f;
    if (on) {
        const float x1 = __fmaf_rn((float)is + 0.5f, 0.5f * g.bx, g.x_d0);
        const float y1 = __fmaf_rn((float)js + 0.5f, 0.5f * g.by, g.y_d0);
        float sm;
        if (trace<0>(G, vol, src.x0, src.y0, src.z0, x1, y1, -g.detectorR, &sm)) {
            v = sm;
            if (sub) sub[((int64_t)blockIdx.z * nby2 + js) * nbx2 + is] = sm;
        }
    }
    tile[ty][tx] = v;
    __syncthreads();
    if (on && ((tx | ty) & 1) == 0) {
        float m = (((tile[ty][tx] + tile[ty][tx + 1]) + tile[ty + 1][tx]) + tile[ty + 1][tx + 1]) *
                  0.25f;
        if (COS) m = m * src.ct;
        out[(int64_t)blockIdx.z * g.nbx * g.nby + bin_off<JI>(g, is >> 1, js >> 1)] = m;
    }
}

// Fused forward projection + h, one block per 32 x 4 bins of one subset view;
// K Siddon steps per gather round.  The walk waits on its volume gathers, so
// residency pays: 12 blocks per SM (40 registers, no spills) run it 5 % faster
// on the clinical workload than the 10 that 48 registers allow (K = 8 needs
// more registers and keeps 8).
template <int K>
__global__ void __launch_bounds__(128, (K >= 8 ? 8 : 12)) fp_h_kernel(const __grid_constant__ Geo G,
                                                   const float* __restrict__ vol,
                                                   float* __restrict__ h,
                                                   const float* __restrict__ angles,
                                                   const int32_t* __restrict__ index, int a0,
                                                   const float* __restrict__ y,
                                                   const float* __restrict__ b,
                                                   const float* __restrict__ r) {
    __shared__ ViewSrc src;
    fp_h_tile<K>(G, vol, h, angles, index, a0, y, b, r, blockIdx.x, blockIdx.y, blockIdx.z, src);
}

// fp_h_kernel with the subset's FP64 data term: one partial per block in red
// (project.cuh, DATA), summed by partials_sum_kernel.
template <int K>
__global__ void __launch_bounds__(128) fp_h_data_kernel(const __grid_constant__ Geo G,
                                                        const float* __restrict__ vol,
                                                        float* __restrict__ h,
                                                        const float* __restrict__ angles,
                                                        const int32_t* __restrict__ index, int a0,
                                                        const float* __restrict__ y,
                                                        const float* __restrict__ b,
                                                        const float* __restrict__ r,
                                                        double* __restrict__ red) {
    __shared__ ViewSrc src;
    fp_h_tile<K, true>(G, vol, h, angles, index, a0, y, b, r, blockIdx.x, blockIdx.y, blockIdx.z,
                       src, red);
}

__global__ void __launch_bounds__(1024) partials_sum_kernel(const double* __restrict__ red,
                                                            int64_t n, double* __restrict__ out) {
    sum_partials(red, n, out);
}

// The same with the volume staged slab by slab through shared memory by TMA
// (slab.cuh); bit-identical to fp_h_kernel.  Measured on the clinical
// workload it is slower than the direct gathers (0.255 ms with 4-plane slabs,
// 0.346 ms with 2-plane slabs, against 0.162 ms): the walk's gathers already
// hit L1 three times in four and the walk is instruction bound, so the
// per-slab synchronisation and bookkeeping cost more than the latency they
// hide.  It is kept as an option (NR_STAGE_TMA).
template <int K, int SZ>
__global__ void __launch_bounds__(128, (SZ >= 4 ? 6 : 10)) fp_h_slab_kernel(
    const __grid_constant__ Geo G, const __grid_constant__ CUtensorMap map,
    const float* __restrict__ vol, float* __restrict__ h, const float* __restrict__ angles,
    const int32_t* __restrict__ index, int a0, const float* __restrict__ y,
    const float* __restrict__ b, const float* __restrict__ r, int* __restrict__ status) {
    extern __shared__ __align__(128) float sbuf[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ ViewSrc src;
    __shared__ SlabBox box[2];
    fp_h_slab_tile<K, SZ>(G, &map, vol, h, angles, index, a0, y, b, r, status, sbuf, src, box,
                          bar);
}

// gamma * yry for every view in one pass (the d precompute's detector term,
// Tomo_OSTR_gold.cpp:183-218), [view][j][i], original view order, identity
// index.  yry = (y-r)^2/y with the reference's guards.
template <int MODE>
__global__ void __launch_bounds__(128) gamma_yry_kernel(const __grid_constant__ Geo G,
                                                        float* __restrict__ out,
                                                        const float* __restrict__ angles,
                                                        const float* __restrict__ y,
                                                        const float* __restrict__ r) {
    __shared__ ViewSrc src;
    const nr_geom& g = G.g;
    const int a = blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[a]);
    __syncthreads();
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nbx || j >= g.nby) return;
    float gam = 0.f;  // gamma buffer is zeroed before the projection (Tomo_OSTR_gold.cpp:441)
    float v;
    if (trace<MODE>(G, nullptr, src.x0, src.y0, src.z0, bin_x(g, i), bin_y(g, j), -g.detectorR, &v))
        gam = v;
    const int64_t o = (int64_t)a * g.nbx * g.nby + bin_off<true>(g, i, j);
    const float yy = y[o];
    float c = 0.f;
    if (yy != 0.f) {
        float dif = yy - (r ? r[o] : 0.f);
        if (dif <= 0.f) dif = yy;
        c = __fdiv_rn(dif * dif, yy);
    }
    out[o] = c * gam;
}

}  // namespace nr

using namespace nr;

static nr_status check_views(const nr_geom* g, const float* angles, const int32_t* index,
                             int32_t a0, int32_t a1) {
    if (!geom_ok(g)) return NR_ERR_BAD_GEOMETRY;
    if (!angles || !index || a0 < 0 || a1 < a0) return NR_ERR_BAD_ARGUMENT;
    if (a1 - a0 > 65535) return NR_ERR_BAD_ARGUMENT;
    return NR_OK;
}

NR_API nr_status nr_fp_ostr(const nr_geom* g, const float* x, float* line, const float* angles,
                            const int32_t* index, int32_t a0, int32_t a1, void* stream) {
    nr_status st = check_views(g, angles, index, a0, a1);
    if (st != NR_OK) return st;
    if (!x || !line) return NR_ERR_BAD_ARGUMENT;
    if (a1 == a0) return NR_OK;
    dim3 blk(32, 4), grd(cdiv(g->nbx, 32), cdiv(g->nby, 4), a1 - a0);
    fp_kernel<0, false><<<grd, blk, 0, as_stream(stream)>>>(make_geo(*g), x, line, angles, index, a0);
    return launch_status();
}

NR_API nr_status nr_fp_gamma(const nr_geom* g, float* gamma, const float* angles,
                             const int32_t* index, int32_t a0, int32_t a1, int32_t mode,
                             void* stream) {
    nr_status st = check_views(g, angles, index, a0, a1);
    if (st != NR_OK) return st;
    if (!gamma || (mode != NR_GAMMA_LENGTH && mode != NR_GAMMA_CHORD)) return NR_ERR_BAD_ARGUMENT;
    if (a1 == a0) return NR_OK;
    dim3 blk(32, 4), grd(cdiv(g->nbx, 32), cdiv(g->nby, 4), a1 - a0);
    if (mode == NR_GAMMA_LENGTH)
        fp_kernel<2, false><<<grd, blk, 0, as_stream(stream)>>>(make_geo(*g), nullptr, gamma,
                                                                angles, index, a0);
    else
        fp_kernel<1, false><<<grd, blk, 0, as_stream(stream)>>>(make_geo(*g), nullptr, gamma,
                                                                angles, index, a0);
    return launch_status();
}

NR_API nr_status nr_fp_sart(const nr_geom* g, const float* x, float* prj_est, float* normprj,
                            const float* angles, const int32_t* index, int32_t a0, int32_t a1,
                            int32_t use_cos, void* stream) {
    nr_status st = check_views(g, angles, index, a0, a1);
    if (st != NR_OK) return st;
    if (!x || !prj_est || !normprj || prj_est == normprj) return NR_ERR_BAD_ARGUMENT;
    if (a1 == a0) return NR_OK;
    dim3 blk(32, 4), grd(cdiv(g->nbx, 32), cdiv(g->nby, 4), a1 - a0);
    if (use_cos)
        fp_sart_kernel<true><<<grd, blk, 0, as_stream(stream)>>>(make_geo(*g), x, prj_est, normprj,
                                                                 angles, index, a0);
    else
        fp_sart_kernel<false><<<grd, blk, 0, as_stream(stream)>>>(make_geo(*g), x, prj_est,
                                                                  normprj, angles, index, a0);
    return launch_status();
}

NR_API nr_status nr_fp_4r(const nr_geom* g, const float* x, float* prj, float* sub,
                          const float* angles, const int32_t* index, int32_t a0, int32_t a1,
                          int32_t use_cos, int32_t layout, void* stream) {
    nr_status st = check_views(g, angles, index, a0, a1);
    if (st != NR_OK) return st;
    if (!x || !prj || prj == sub || (layout != NR_LAYOUT_IJ && layout != NR_LAYOUT_JI))
        return NR_ERR_BAD_ARGUMENT;
    if ((int64_t)4 * g->nbx * g->nby * (a1 - a0) >= (int64_t)1 << 31) return NR_ERR_BAD_GEOMETRY;
    if (a1 == a0) return NR_OK;
    dim3 blk(32, 8), grd(cdiv(2 * (int64_t)g->nbx, 32), cdiv(2 * (int64_t)g->nby, 8), a1 - a0);
    const Geo G = make_geo(*g);
    cudaStream_t s = as_stream(stream);
    if (use_cos) {
        if (layout == NR_LAYOUT_JI)
            fp_4r_kernel<true, true><<<grd, blk, 0, s>>>(G, x, prj, sub, angles, index, a0);
        else
            fp_4r_kernel<true, false><<<grd, blk, 0, s>>>(G, x, prj, sub, angles, index, a0);
    } else {
        if (layout == NR_LAYOUT_JI)
            fp_4r_kernel<false, true><<<grd, blk, 0, s>>>(G, x, prj, sub, angles, index, a0);
        else
            fp_4r_kernel<false, false><<<grd, blk, 0, s>>>(G, x, prj, sub, angles, index, a0);
    }
    return launch_status();
}

// Internal launchers used by the device-resident path (ostr.cu).
namespace nr {

// cuTensorMapEncodeTiled from the driver, looked up once.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
        }
        return (PFN_cuTensorMapEncodeTiled_v12000)p;
    }();
    return fn;
}

// The same entry point for the other translation units (cnn.cu).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encode_fn() { return tensor_map_encoder(); }

#ifndef NR_SLAB_Z
#define NR_SLAB_Z 4
#endif
constexpr int SLAB_Z = NR_SLAB_Z;  // planes per staged slab

// The TMA descriptor of volume x ([z][y][x] float) with the staging box; false
// when the volume cannot be described (x rows not a multiple of 16 bytes,
// misaligned base, no driver entry point).
bool slab_map(const nr_geom& g, const float* x, CUtensorMap* map) {
    if (g.nx % 4 != 0 || ((uintptr_t)x & 15) != 0) return false;
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)g.nx * 4, (cuuint64_t)g.nx * g.ny * 4};
    const cuuint32_t box[3] = {SLAB_FX, SLAB_FY, SLAB_Z};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)x, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The TMA descriptor of volume x with a box of bx x by x bz voxels (bx a
// multiple of 4) whose out-of-volume elements read as NaN: the update's
// planes with their halo (update.cuh), where NaN marks a neighbour outside
// the volume.  False when the volume cannot be described.
bool volume_map_nan(const nr_geom& g, const float* x, int bx, int by, int bz, CUtensorMap* map) {
    if (g.nx % 4 != 0 || bx % 4 != 0 || ((uintptr_t)x & 15) != 0) return false;
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)g.nx * 4, (cuuint64_t)g.nx * g.ny * 4};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)x, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NAN_REQUEST_ZERO_FMA) == CUDA_SUCCESS;
}

// premap: x's descriptor when the caller encoded it already (slab_map), else
// nullptr (encoded here when staging applies).
nr_status launch_fp_h(const nr_geom& g, int k, int stage, const float* x, float* h,
                      const float* angles, const int32_t* index, int a0, int nviews,
                      const float* y, const float* b, const float* r, int* status,
                      const CUtensorMap* premap, cudaStream_t st) {
    dim3 blk(32, 4), grd(cdiv(g.nbx, 32), cdiv(g.nby, 4), nviews);
    const Geo G = make_geo(g);
    CUtensorMap map;
    bool staged = false;
    if (stage == NR_STAGE_TMA && k != 8) {
        if (premap) {
            map = *premap;
            staged = true;
        } else {
            staged = slab_map(g, x, &map);
        }
    }
    if (staged) {
        const size_t smem = 2 * SlabCfg<SLAB_Z>::BYTES;
        if (k == 2)
            fp_h_slab_kernel<2, SLAB_Z><<<grd, blk, smem, st>>>(G, map, x, h, angles, index, a0,
                                                                y, b, r, status);
        else
            fp_h_slab_kernel<4, SLAB_Z><<<grd, blk, smem, st>>>(G, map, x, h, angles, index, a0,
                                                                y, b, r, status);
        return launch_status();
    }
    if (k == 2)
        fp_h_kernel<2><<<grd, blk, 0, st>>>(G, x, h, angles, index, a0, y, b, r);
    else if (k == 8)
        fp_h_kernel<8><<<grd, blk, 0, st>>>(G, x, h, angles, index, a0, y, b, r);
    else
        fp_h_kernel<4><<<grd, blk, 0, st>>>(G, x, h, angles, index, a0, y, b, r);
    return launch_status();
}

// The fused projection of launch_fp_h (direct gathers, K steps per round)
// with the subset's FP64 data term into out[0]; red holds red_n partials.
nr_status launch_fp_h_data(const nr_geom& g, int k, const float* x, float* h,
                           const float* angles, const int32_t* index, int a0, int nviews,
                           const float* y, const float* b, const float* r, double* red,
                           int64_t red_n, double* out, cudaStream_t st) {
    dim3 blk(32, 4), grd(cdiv(g.nbx, 32), cdiv(g.nby, 4), nviews);
    const int64_t n = (int64_t)grd.x * grd.y * grd.z;
    if (n > red_n) return NR_ERR_WORKSPACE;
    const Geo G = make_geo(g);
    if (k == 2)
        fp_h_data_kernel<2><<<grd, blk, 0, st>>>(G, x, h, angles, index, a0, y, b, r, red);
    else if (k == 8)
        fp_h_data_kernel<8><<<grd, blk, 0, st>>>(G, x, h, angles, index, a0, y, b, r, red);
    else
        fp_h_data_kernel<4><<<grd, blk, 0, st>>>(G, x, h, angles, index, a0, y, b, r, red);
    partials_sum_kernel<<<1, 1024, 0, st>>>(red, n, out);
    return launch_status();
}

nr_status launch_fp_ji(const nr_geom& g, const float* x, float* line, const float* angles,
                       const int32_t* index, int a0, int nviews, cudaStream_t st) {
    dim3 blk(32, 4), grd(cdiv(g.nbx, 32), cdiv(g.nby, 4), nviews);
    fp_kernel<0, true><<<grd, blk, 0, st>>>(make_geo(g), x, line, angles, index, a0);
    return launch_status();
}

nr_status launch_gamma_yry(const nr_geom& g, int gamma_mode, float* out, const float* angles,
                           const float* y, const float* r, cudaStream_t st) {
    dim3 blk(32, 4), grd(cdiv(g.nbx, 32), cdiv(g.nby, 4), g.n_angles);
    if (gamma_mode == NR_GAMMA_CHORD)
        gamma_yry_kernel<1><<<grd, blk, 0, st>>>(make_geo(g), out, angles, y, r);
    else
        gamma_yry_kernel<2><<<grd, blk, 0, st>>>(make_geo(g), out, angles, y, r);
    return launch_status();
}

}  // namespace nr
