// sart.cu -- the device-resident OS-SART loop.
//
// The reference ships the SART / OS-SART kernels (Tomo_OSTR.cu:1177-1311,
// 1737-2183) and their launch wrappers (:2249-2332, 2460-2558) but leaves the
// driver empty (Recon_Method 3, Tomo_OSTR_gold.cpp:1523-1525).  This file is
// that driver, in the order the kernels compose: per subset of views
//     FP_SART(x) -> diff = (p - FP) / normprj -> x += lambda BP_OSSART(diff)
// (plus prior_GPU_SART and backprj_OSSART_R for the regularised form), with
// the subset order of the OSTR driver (Tomo_OSTR_gold.cpp:628-642).
//
// Two launches per sub-iteration:
//   sart_fp_diff_kernel  one thread per subset bin: Siddon sum, the
//                        difference against the stored line integral, divided
//                        by the ray's chord (0 where the chord is 0); with
//                        supersample, sart_fp_diff_4r_kernel does the same on
//                        the mean of 2 x 2 sub-rays per bin (nr_fp_4r's
//                        projector) against their mean chord
//   sart_update_kernel   the fused update tile of update.cuh in its OS-SART
//                        kinds: sensitivity-normalised back projection, the
//                        hyperbola prior from the 3-plane ring, the step and
//                        the clamp, written to the second volume buffer
// normprj -- the in-volume chord of each ray -- does not depend on x, so it
// is traced once at set-up (the reference re-traces it with every FP).
//
// Workspace (caller-allocated, 256-byte aligned sections; the status word
// first, so nr_ostr_check reads it as for OSTR):
//   status int32[64]
//   index  int32[A]                   view order (subset-major)
//   angles float[A]
//   p      float[A][BINSy][BINSx]     line integrals, subset order, i fastest
//   norm   float[A][BINSy][BINSx]     chord lengths, same layout
//   diff   float[Vs][BINSy][BINSx]    the subset's normalised difference
//   xtmp   float[N]                   second volume buffer (ping-pong)
//   bpx, bpy float4[A][nz][nx], [A][nz][ny]  back-projection tables (update.cuh)
#include "project.cuh"
#include "update.cuh"

namespace nr {

nr_status launch_subset_index(int32_t* idx, const float* angles_in, float* angles_out, int A,
                              int M, cudaStream_t s);
nr_status launch_clear_status(int* status, cudaStream_t s);
nr_status launch_transpose(float* out, const float* in, int rows, int cols, int nviews, int M,
                           int Vs, cudaStream_t st);
nr_status launch_bp_tables(const nr_geom& g, const float* angles, const int32_t* index,
                           float4* tx, float4* ty, cudaStream_t st);

namespace {

struct SartLayout {
    size_t status, index, angles, p, norm, diff, xtmp, bpx, bpy, total;
};

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

SartLayout sart_layout(const nr_geom& g, const nr_sart_params& p) {
    const int64_t A = g.n_angles, B = (int64_t)g.nbx * g.nby;
    const int64_t N = (int64_t)g.nx * g.ny * g.nz;
    const int64_t Vs = A / p.subset_num;
    SartLayout L;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    L.status = take(64 * sizeof(int32_t));
    L.index = take(A * sizeof(int32_t));
    L.angles = take(A * sizeof(float));
    L.p = take(A * B * sizeof(float));
    L.norm = take(A * B * sizeof(float));
    L.diff = take((Vs * B + bp_pad(g)) * sizeof(float));  // + zeros the tap pairs may reach
    L.xtmp = take(N * sizeof(float));
    L.bpx = take((size_t)A * g.nz * g.nx * sizeof(float4));
    L.bpy = take((size_t)A * g.nz * g.ny * sizeof(float4));
    L.total = o;
    return L;
}

struct SartWS {
    int* status;
    int32_t* index;
    float *angles, *p, *norm, *diff, *xtmp;
    float4 *bpx, *bpy;
};

SartWS sart_carve(void* base, const SartLayout& L) {
    char* c = (char*)base;
    SartWS w;
    w.status = (int*)(c + L.status);
    w.index = (int32_t*)(c + L.index);
    w.angles = (float*)(c + L.angles);
    w.p = (float*)(c + L.p);
    w.norm = (float*)(c + L.norm);
    w.diff = (float*)(c + L.diff);
    w.xtmp = (float*)(c + L.xtmp);
    w.bpx = (float4*)(c + L.bpx);
    w.bpy = (float4*)(c + L.bpy);
    return w;
}

nr_status sart_check_params(const nr_geom* g, const nr_sart_params* p) {
    if (!geom_ok(g)) return NR_ERR_BAD_GEOMETRY;
    if (!p) return NR_ERR_BAD_ARGUMENT;
    if (p->subset_num <= 0 || g->n_angles % p->subset_num != 0) return NR_ERR_BAD_GEOMETRY;
    if (g->n_angles / p->subset_num > UPD_VIEWS_SMEM) return NR_ERR_BAD_ARGUMENT;
    if (!(fabsf(p->lambda) < INFINITY) || !(fabsf(p->beta) < INFINITY)) return NR_ERR_BAD_ARGUMENT;
    if (p->regularized && (p->delta == 0.f || !(fabsf(p->delta) < INFINITY)))
        return NR_ERR_BAD_ARGUMENT;  // prior_GPU_SART exits on delta == 0 (Tomo_OSTR.cu:2260)
    if (p->fp_batch != 0 && p->fp_batch != 2 && p->fp_batch != 4 && p->fp_batch != 8)
        return NR_ERR_BAD_ARGUMENT;
    if (p->upd_planes != 0 && p->upd_planes != 8 && p->upd_planes != 16 && p->upd_planes != 32)
        return NR_ERR_BAD_ARGUMENT;
    if (p->supersample != 0 && p->supersample != 1) return NR_ERR_BAD_ARGUMENT;
    if (g->ny > 65535 || g->nz > 65535 || g->n_angles > 65535) return NR_ERR_BAD_GEOMETRY;
    if (!bp_tables_fit(*g)) return NR_ERR_BAD_GEOMETRY;
    return NR_OK;
}

nr_status sart_check_ws(const nr_geom* g, const nr_sart_params* p, void* ws, size_t bytes,
                        SartLayout* L) {
    nr_status st = sart_check_params(g, p);
    if (st != NR_OK) return st;
    *L = sart_layout(*g, *p);
    if (!ws || bytes < L->total || ((uintptr_t)ws & 255) != 0) return NR_ERR_WORKSPACE;
    return NR_OK;
}

}  // namespace

// Chord of every ray, all views in subset order, [view][j][i]; 0 for rays
// that miss the volume (so their difference is 0).
__global__ void __launch_bounds__(128) sart_norm_kernel(const __grid_constant__ Geo G,
                                                        float* __restrict__ norm,
                                                        const float* __restrict__ angles,
                                                        const int32_t* __restrict__ index) {
    __shared__ ViewSrc src;
    const nr_geom& g = G.g;
    const int a = blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nbx || j >= g.nby) return;
    float v;
    if (!trace<1>(G, nullptr, src.x0, src.y0, src.z0, bin_x(g, i), bin_y(g, j), -g.detectorR, &v))
        v = 0.f;
    norm[(int64_t)a * g.nbx * g.nby + bin_off<true>(g, i, j)] = v;
}

// diff = (p - FP(x) [cos]) / norm for the subset views [a0, a0 + gridDim.z);
// 12 resident blocks per SM, as fp_h_kernel.
template <int K, bool COS>
__global__ void __launch_bounds__(128, (K >= 8 ? 8 : 12)) sart_fp_diff_kernel(
    const __grid_constant__ Geo G, const float* __restrict__ vol, float* __restrict__ diff,
    const float* __restrict__ angles, const int32_t* __restrict__ index, int a0,
    const float* __restrict__ p, const float* __restrict__ norm) {
    __shared__ ViewSrc src;
    const nr_geom& g = G.g;
    const int a = a0 + blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nbx || j >= g.nby) return;
    const int64_t B = (int64_t)g.nbx * g.nby;
    const int64_t off = bin_off<true>(g, i, j);
    const float nv = norm[(int64_t)a * B + off];
    float out = 0.f;
    if (nv != 0.f) {
        float v = 0.f;
        trace<0, K>(G, vol, src.x0, src.y0, src.z0, bin_x(g, i), bin_y(g, j), -g.detectorR, &v);
        const float est = COS ? v * src.ct : v;
        out = __fdiv_rn(p[(int64_t)a * B + off] - est, nv);
    }
    diff[(int64_t)blockIdx.z * B + off] = out;
}

// The 2 x 2 super-sampled forms (supersample = 1; the projector of nr_fp_4r):
// one thread per sub-ray, 32 x 8 sub-rays = 16 x 4 bins per block, the four
// sub-rays of a bin merged in shared memory in the order of nr_fp_4r.
// MODE 1 traces chords (set-up), MODE 0 line integrals.
template <int MODE>
__device__ __forceinline__ bool sub_ray_merge(const Geo& G, const float* __restrict__ vol,
                                              const ViewSrc& src, float (*tile)[33], float* m,
                                              int* i, int* j) {
    const nr_geom& g = G.g;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int is = blockIdx.x * 32 + tx, js = blockIdx.y * 8 + ty;
    const bool on = is < 2 * g.nbx && js < 2 * g.nby;
    float v = 0.f;
    if (on) {
        const float x1 = __fmaf_rn((float)is + 0.5f, 0.5f * g.bx, g.x_d0);
        const float y1 = __fmaf_rn((float)js + 0.5f, 0.5f * g.by, g.y_d0);
        float t;
        if (trace<MODE>(G, vol, src.x0, src.y0, src.z0, x1, y1, -g.detectorR, &t)) v = t;
    }
    tile[ty][tx] = v;
    __syncthreads();
    if (!on || ((tx | ty) & 1) != 0) return false;
    *m = (((tile[ty][tx] + tile[ty][tx + 1]) + tile[ty + 1][tx]) + tile[ty + 1][tx + 1]) * 0.25f;
    *i = is >> 1;
    *j = js >> 1;
    return true;
}

__global__ void __launch_bounds__(256) sart_norm_4r_kernel(const __grid_constant__ Geo G,
                                                           float* __restrict__ norm,
                                                           const float* __restrict__ angles,
                                                           const int32_t* __restrict__ index) {
    __shared__ ViewSrc src;
    __shared__ float tile[8][33];
    const nr_geom& g = G.g;
    const int a = blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    float m;
    int i, j;
    if (sub_ray_merge<1>(G, nullptr, src, tile, &m, &i, &j))
        norm[(int64_t)a * g.nbx * g.nby + bin_off<true>(g, i, j)] = m;
}

template <bool COS>
__global__ void __launch_bounds__(256) sart_fp_diff_4r_kernel(
    const __grid_constant__ Geo G, const float* __restrict__ vol, float* __restrict__ diff,
    const float* __restrict__ angles, const int32_t* __restrict__ index, int a0,
    const float* __restrict__ p, const float* __restrict__ norm) {
    __shared__ ViewSrc src;
    __shared__ float tile[8][33];
    const nr_geom& g = G.g;
    const int a = a0 + blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    float m;
    int i, j;
    if (!sub_ray_merge<0>(G, vol, src, tile, &m, &i, &j)) return;
    const int64_t B = (int64_t)g.nbx * g.nby;
    const int64_t off = bin_off<true>(g, i, j);
    const float nv = norm[(int64_t)a * B + off];
    const float est = COS ? m * src.ct : m;
    diff[(int64_t)blockIdx.z * B + off] = nv != 0.f ? __fdiv_rn(p[(int64_t)a * B + off] - est, nv)
                                                    : 0.f;
}

template <int KIND, int ZC, int NV>
__global__ void __launch_bounds__(256, NV == 1 ? 8 : 0) sart_update_kernel(
    const __grid_constant__ Geo G, const __grid_constant__ PriorW5 W,
    const float* __restrict__ x, float* __restrict__ x_out, const float* __restrict__ diff,
    const float* __restrict__ angles, const int32_t* __restrict__ index,
    const __grid_constant__ BpTab T, int a0, int nv, float lambda, float beta, float delta,
    int* __restrict__ status) {
    __shared__ UpdSmem sm;
    update_tile<NR_POT_HYPERBOLA, ZC, KIND, NV>(G, W, x, x_out, nullptr, diff, angles, index, T,
                                                a0, nv, lambda, beta, delta, status, blockIdx.x,
                                                blockIdx.y, blockIdx.z, sm);
}

namespace {

template <bool COS>
nr_status launch_fp_diff_c(const nr_geom& g, int k, const float* x, const SartWS& w, int a0,
                           int nv, bool ss, cudaStream_t s) {
    const Geo G = make_geo(g);
    if (ss) {
        dim3 blk(32, 8), grd(cdiv(2 * (int64_t)g.nbx, 32), cdiv(2 * (int64_t)g.nby, 8), nv);
        sart_fp_diff_4r_kernel<COS><<<grd, blk, 0, s>>>(G, x, w.diff, w.angles, w.index, a0, w.p,
                                                         w.norm);
        return launch_status();
    }
    dim3 blk(32, 4), grd(cdiv(g.nbx, 32), cdiv(g.nby, 4), nv);
    if (k == 2)
        sart_fp_diff_kernel<2, COS><<<grd, blk, 0, s>>>(G, x, w.diff, w.angles, w.index, a0, w.p,
                                                        w.norm);
    else if (k == 8)
        sart_fp_diff_kernel<8, COS><<<grd, blk, 0, s>>>(G, x, w.diff, w.angles, w.index, a0, w.p,
                                                        w.norm);
    else
        sart_fp_diff_kernel<4, COS><<<grd, blk, 0, s>>>(G, x, w.diff, w.angles, w.index, a0, w.p,
                                                        w.norm);
    return launch_status();
}

template <int KIND, int ZC>
nr_status launch_sart_update_t(const nr_geom& g, const nr_sart_params& p, const float* x,
                               float* x_out, const SartWS& w, int a0, int nv, cudaStream_t s) {
    dim3 blk(UTX, UTY), grd(cdiv(g.nx, UTX), cdiv(g.ny, UTY), cdiv(g.nz, ZC));
    // unit neighbour distances: G_Huber_prior has no z ratio (Tomo_OSTR.cu:303)
    const float delta = p.regularized ? p.delta : 1.f;
    const Geo G = make_geo(g);
    const PriorW5 W = make_w5(1.f, delta);
    const BpTab T{w.bpx, w.bpy};
    if (nv == 1)
        sart_update_kernel<KIND, ZC, 1><<<grd, blk, 0, s>>>(G, W, x, x_out, w.diff, w.angles,
                                                            w.index, T, a0, nv, p.lambda, p.beta,
                                                            delta, w.status);
    else
        sart_update_kernel<KIND, ZC, 0><<<grd, blk, 0, s>>>(G, W, x, x_out, w.diff, w.angles,
                                                            w.index, T, a0, nv, p.lambda, p.beta,
                                                            delta, w.status);
    return launch_status();
}

template <int KIND>
nr_status launch_sart_update_z(const nr_geom& g, const nr_sart_params& p, const float* x,
                               float* x_out, const SartWS& w, int a0, int nv, cudaStream_t s) {
    switch (p.upd_planes) {
    case 8: return launch_sart_update_t<KIND, 8>(g, p, x, x_out, w, a0, nv, s);
    case 32: return launch_sart_update_t<KIND, 32>(g, p, x, x_out, w, a0, nv, s);
    default: return launch_sart_update_t<KIND, 16>(g, p, x, x_out, w, a0, nv, s);
    }
}

nr_status sart_project(const nr_geom& g, const nr_sart_params& p, const float* x, int subset,
                       const SartWS& w, cudaStream_t s) {
    const int Vs = g.n_angles / p.subset_num, a0 = subset * Vs;
    return p.use_cos ? launch_fp_diff_c<true>(g, p.fp_batch, x, w, a0, Vs, p.supersample, s)
                     : launch_fp_diff_c<false>(g, p.fp_batch, x, w, a0, Vs, p.supersample, s);
}

nr_status sart_update(const nr_geom& g, const nr_sart_params& p, const float* x, float* x_out,
                      int subset, const SartWS& w, cudaStream_t s) {
    const int Vs = g.n_angles / p.subset_num, a0 = subset * Vs;
    return p.regularized ? launch_sart_update_z<UPD_SART_R>(g, p, x, x_out, w, a0, Vs, s)
                         : launch_sart_update_z<UPD_SART>(g, p, x, x_out, w, a0, Vs, s);
}

// One sub-iteration: x -> x_out (x_out != x).
nr_status sart_step(const nr_geom& g, const nr_sart_params& p, const float* x, float* x_out,
                    int subset, const SartWS& w, cudaStream_t s) {
    nr_status st = sart_project(g, p, x, subset, w, s);
    if (st != NR_OK) return st;
    return sart_update(g, p, x, x_out, subset, w, s);
}

nr_status sart_enqueue(const nr_geom& g, const nr_sart_params& p, float* x, int n_iters,
                       const SartWS& w, cudaStream_t s) {
    const int64_t N = (int64_t)g.nx * g.ny * g.nz;
    float* cur = x;
    float* nxt = w.xtmp;
    for (int it = 0; it < n_iters; it++)
        for (int a = 0; a < p.subset_num; a++) {
            nr_status st = sart_step(g, p, cur, nxt, a, w, s);
            if (st != NR_OK) return st;
            float* t = cur;
            cur = nxt;
            nxt = t;
        }
    if (cur != x &&
        cudaMemcpyAsync(x, cur, N * sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return NR_ERR_CUDA;
    return NR_OK;
}

}  // namespace
}  // namespace nr

using namespace nr;

NR_API nr_status nr_sart_workspace_size(const nr_geom* g, const nr_sart_params* p,
                                        size_t* bytes) {
    nr_status st = sart_check_params(g, p);
    if (st != NR_OK) return st;
    if (!bytes) return NR_ERR_BAD_ARGUMENT;
    *bytes = sart_layout(*g, *p).total;
    return NR_OK;
}

NR_API nr_status nr_sart_setup(const nr_geom* g, const nr_sart_params* p, const float* angles,
                               const float* line, void* workspace, size_t ws_bytes,
                               void* stream) {
    SartLayout L;
    nr_status st = sart_check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!angles || !line) return NR_ERR_BAD_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    SartWS w = sart_carve(workspace, L);
    const int A = g->n_angles, M = p->subset_num, Vs = A / M;
    if ((st = launch_clear_status(w.status, s)) != NR_OK) return st;
    if ((st = launch_subset_index(w.index, angles, w.angles, A, M, s)) != NR_OK) return st;
    if ((st = launch_bp_tables(*g, w.angles, w.index, w.bpx, w.bpy, s)) != NR_OK) return st;
    if (cudaMemsetAsync(w.diff + (int64_t)Vs * g->nbx * g->nby, 0, bp_pad(*g) * sizeof(float),
                        s) != cudaSuccess)
        return NR_ERR_CUDA;
    // [view][i][j] original order -> [view][j][i] subset order.
    if ((st = launch_transpose(w.p, line, g->nbx, g->nby, A, M, Vs, s)) != NR_OK) return st;
    if (p->supersample) {
        dim3 blk(32, 8), grd(cdiv(2 * (int64_t)g->nbx, 32), cdiv(2 * (int64_t)g->nby, 8), A);
        sart_norm_4r_kernel<<<grd, blk, 0, s>>>(make_geo(*g), w.norm, w.angles, w.index);
    } else {
        dim3 blk(32, 4), grd(cdiv(g->nbx, 32), cdiv(g->nby, 4), A);
        sart_norm_kernel<<<grd, blk, 0, s>>>(make_geo(*g), w.norm, w.angles, w.index);
    }
    return launch_status();
}

NR_API nr_status nr_sart_project(const nr_geom* g, const nr_sart_params* p, const float* x,
                                 int32_t subset, void* workspace, size_t ws_bytes, void* stream) {
    SartLayout L;
    nr_status st = sart_check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || subset < 0 || subset >= p->subset_num) return NR_ERR_BAD_ARGUMENT;
    return sart_project(*g, *p, x, subset, sart_carve(workspace, L), as_stream(stream));
}

NR_API nr_status nr_sart_update(const nr_geom* g, const nr_sart_params* p, const float* x,
                                float* x_out, int32_t subset, void* workspace, size_t ws_bytes,
                                void* stream) {
    SartLayout L;
    nr_status st = sart_check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || !x_out || x == x_out || subset < 0 || subset >= p->subset_num)
        return NR_ERR_BAD_ARGUMENT;
    return sart_update(*g, *p, x, x_out, subset, sart_carve(workspace, L), as_stream(stream));
}

NR_API nr_status nr_sart_subiter(const nr_geom* g, const nr_sart_params* p, float* x,
                                 int32_t subset, void* workspace, size_t ws_bytes, void* stream) {
    SartLayout L;
    nr_status st = sart_check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || subset < 0 || subset >= p->subset_num) return NR_ERR_BAD_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    SartWS w = sart_carve(workspace, L);
    const int64_t N = (int64_t)g->nx * g->ny * g->nz;
    if ((st = sart_step(*g, *p, x, w.xtmp, subset, w, s)) != NR_OK) return st;
    if (cudaMemcpyAsync(x, w.xtmp, N * sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return NR_ERR_CUDA;
    return NR_OK;
}

NR_API nr_status nr_sart_iterate(const nr_geom* g, const nr_sart_params* p, float* x,
                                 int32_t n_iters, void* workspace, size_t ws_bytes,
                                 void* stream) {
    SartLayout L;
    nr_status st = sart_check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || n_iters < 0) return NR_ERR_BAD_ARGUMENT;
    return sart_enqueue(*g, *p, x, n_iters, sart_carve(workspace, L), as_stream(stream));
}

NR_API nr_status nr_sart_graph_create(const nr_geom* g, const nr_sart_params* p, float* x,
                                      int32_t n_iters, void* workspace, size_t ws_bytes,
                                      void* stream, void** graph) {
    SartLayout L;
    nr_status st = sart_check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || n_iters < 1 || !graph || !stream) return NR_ERR_BAD_ARGUMENT;
    *graph = nullptr;
    cudaStream_t s = as_stream(stream);
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return NR_ERR_CUDA;
    st = sart_enqueue(*g, *p, x, n_iters, sart_carve(workspace, L), s);
    return finish_capture(s, st, graph);
}

NR_API nr_status nr_sart_workspace_section(const nr_geom* g, const nr_sart_params* p,
                                           int32_t section, void* workspace, size_t ws_bytes,
                                           void** ptr, size_t* bytes) {
    SartLayout L;
    nr_status st = sart_check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!ptr || !bytes) return NR_ERR_BAD_ARGUMENT;
    SartWS w = sart_carve(workspace, L);
    const int64_t A = g->n_angles, B = (int64_t)g->nbx * g->nby;
    switch (section) {
    case NR_SART_WS_LINE: *ptr = w.p; *bytes = A * B * sizeof(float); break;
    case NR_SART_WS_NORM: *ptr = w.norm; *bytes = A * B * sizeof(float); break;
    case NR_SART_WS_DIFF: *ptr = w.diff; *bytes = (A / p->subset_num) * B * sizeof(float); break;
    case NR_SART_WS_INDEX: *ptr = w.index; *bytes = A * sizeof(int32_t); break;
    default: return NR_ERR_BAD_ARGUMENT;
    }
    return NR_OK;
}
