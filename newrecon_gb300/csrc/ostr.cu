// ostr.cu -- the device-resident OSTR driver: workspace layout, scan setup
// (regroup + transpose, gamma*yry, curvature d), the subset loop, the FP64
// objective and the status word.
//
// Workspace (caller-allocated, 256-byte aligned sections):
//   status   int32[64]                  device status word (NR_FLAG_*)
//   red      double[red_n]              per-block partial sums of the objective
//   index    int32[A]                   view order (subset-major)
//   angles   float[A]
//   y, b, r  float[A][BINSy][BINSx]     scan in subset order, detector i fastest
//   d        float[N]                   curvature denominators
//   xtmp     float[N]                   second volume buffer (ping-pong)
//   h        float[Vs][BINSy][BINSx]    subset gradient in the detector domain
//   bpx, bpy float4[A][nz][nx], [A][nz][ny]  back-projection tables (update.cuh)
//   gc       float[A][BINSy][BINSx]     gamma*yry (setup only)
//   gr       float[A][BINSy][BINSx]     scatter in original order (setup only; with scatter)
#include <cuda.h>

#include "update.cuh"

namespace nr {

nr_status launch_fp_h(const nr_geom& g, int k, int stage, const float* x, float* h,
                      const float* angles, const int32_t* index, int a0, int nviews,
                      const float* y, const float* b, const float* r, int* status,
                      const CUtensorMap* premap, cudaStream_t st);
bool slab_map(const nr_geom& g, const float* x, CUtensorMap* map);
nr_status launch_gamma_yry(const nr_geom& g, int gamma_mode, float* out, const float* angles,
                           const float* y, const float* r, cudaStream_t st);
nr_status launch_bp(const nr_geom& g, bool ji, float* vol, const float* prj, const float* angles,
                    const int32_t* index, int a0, int nv, cudaStream_t st);
nr_status launch_update(const nr_geom& g, int pot, int zc, int tile, const float* x, float* x_out,
                        const float* d, const float* h, const float* angles, const int32_t* index,
                        const BpTab& T, int a0, int nv, float M, float beta, float delta,
                        int* status, const CUtensorMap* map, cudaStream_t st);
bool volume_map_nan(const nr_geom& g, const float* x, int bx, int by, int bz, CUtensorMap* map);

// The TMA descriptor the update's NR_TILE_TMA form reads volume x through
// (its planes with halo, NaN outside the volume); false when the volume
// cannot be described (IMGSIZx not a multiple of 4, x not 16-byte aligned),
// and the update then runs the one-voxel tile instead.
static bool update_map(const nr_geom& g, const nr_ostr_params& p, const float* x,
                       CUtensorMap* map) {
    return p.upd_tile == NR_TILE_TMA && volume_map_nan(g, x, UTW, USH, 1, map);
}
nr_status launch_bp_tables(const nr_geom& g, const float* angles, const int32_t* index,
                           float4* tx, float4* ty, cudaStream_t st);
nr_status launch_transpose(float* out, const float* in, int rows, int cols, int nviews, int M,
                           int Vs, cudaStream_t st);
nr_status launch_objective(const nr_geom& g, int pot, float delta, const float* x,
                           const float* angles, const int32_t* index, const float* y,
                           const float* b, const float* r, double* red, int64_t red_n,
                           double* out, cudaStream_t st);
int64_t objective_partials(const nr_geom& g);
nr_status launch_fp_h_data(const nr_geom& g, int k, const float* x, float* h,
                           const float* angles, const int32_t* index, int a0, int nviews,
                           const float* y, const float* b, const float* r, double* red,
                           int64_t red_n, double* out, cudaStream_t st);
nr_status launch_penalty(const nr_geom& g, int pot, float delta, const float* x, double* red,
                         int64_t red_n, double* out, cudaStream_t st);

struct Layout {
    size_t status, red, index, angles, y, b, r, d, xtmp, h, bpx, bpy, gc, gr, total;
    int64_t red_n;
};

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

static Layout layout(const nr_geom& g, const nr_ostr_params& p) {
    const int64_t A = g.n_angles, B = (int64_t)g.nbx * g.nby;
    const int64_t N = (int64_t)g.nx * g.ny * g.nz;
    const int64_t Vs = A / p.subset_num;
    Layout L;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    L.red_n = objective_partials(g);
    L.status = take(64 * sizeof(int32_t));
    L.red = take((size_t)L.red_n * sizeof(double));
    L.index = take(A * sizeof(int32_t));
    L.angles = take(A * sizeof(float));
    L.y = take(A * B * sizeof(float));
    L.b = take(A * B * sizeof(float));
    L.r = p.has_scatter ? take(A * B * sizeof(float)) : (size_t)-1;
    L.d = take(N * sizeof(float));
    L.xtmp = take(N * sizeof(float));
    L.h = take((Vs * B + bp_pad(g)) * sizeof(float));  // + zeros the tap pairs may reach
    L.bpx = take((size_t)A * g.nz * g.nx * sizeof(float4));
    L.bpy = take((size_t)A * g.nz * g.ny * sizeof(float4));
    L.gc = take(A * B * sizeof(float));
    L.gr = p.has_scatter ? take(A * B * sizeof(float)) : (size_t)-1;
    L.total = o;
    return L;
}

struct WS {
    int* status;
    double* red;
    int32_t* index;
    float *angles, *y, *b, *r, *d, *xtmp, *h, *gc, *gr;
    float4 *bpx, *bpy;
    int64_t red_n;
    BpTab tab() const { return BpTab{bpx, bpy}; }
};

static WS carve(void* base, const Layout& L) {
    char* c = (char*)base;
    WS w;
    w.status = (int*)(c + L.status);
    w.red = (double*)(c + L.red);
    w.index = (int32_t*)(c + L.index);
    w.angles = (float*)(c + L.angles);
    w.y = (float*)(c + L.y);
    w.b = (float*)(c + L.b);
    w.r = L.r == (size_t)-1 ? nullptr : (float*)(c + L.r);
    w.d = (float*)(c + L.d);
    w.xtmp = (float*)(c + L.xtmp);
    w.h = (float*)(c + L.h);
    w.bpx = (float4*)(c + L.bpx);
    w.bpy = (float4*)(c + L.bpy);
    w.gc = (float*)(c + L.gc);
    w.gr = L.gr == (size_t)-1 ? nullptr : (float*)(c + L.gr);
    w.red_n = L.red_n;
    return w;
}

static nr_status check_params(const nr_geom* g, const nr_ostr_params* p) {
    if (!geom_ok(g)) return NR_ERR_BAD_GEOMETRY;
    if (!p) return NR_ERR_BAD_ARGUMENT;
    if (p->subset_num <= 0 || g->n_angles % p->subset_num != 0) return NR_ERR_BAD_GEOMETRY;
    if (g->vx != g->vy) return NR_ERR_BAD_GEOMETRY;  // Tomo_OSTR_gold.cpp:380-386
    if (p->potential < NR_POT_Q2 || p->potential > NR_POT_HUBER) return NR_ERR_BAD_ARGUMENT;
    if (p->potential != NR_POT_Q2 && !(p->delta > 0.f)) return NR_ERR_BAD_ARGUMENT;
    if (p->gamma_mode != NR_GAMMA_LENGTH && p->gamma_mode != NR_GAMMA_CHORD)
        return NR_ERR_BAD_ARGUMENT;
    if (!(p->beta >= 0.f)) return NR_ERR_BAD_ARGUMENT;
    if (g->n_angles / p->subset_num > 32) return NR_ERR_BAD_ARGUMENT;  // views per subset in smem
    if (p->fp_batch != 0 && p->fp_batch != 2 && p->fp_batch != 4 && p->fp_batch != 8)
        return NR_ERR_BAD_ARGUMENT;
    if (p->upd_planes != 0 && p->upd_planes != 8 && p->upd_planes != 16 && p->upd_planes != 32)
        return NR_ERR_BAD_ARGUMENT;
    if (p->fp_stage != NR_STAGE_OFF && p->fp_stage != NR_STAGE_TMA) return NR_ERR_BAD_ARGUMENT;
    if (p->upd_tile != NR_TILE_1 && p->upd_tile != NR_TILE_2 && p->upd_tile != NR_TILE_TMA)
        return NR_ERR_BAD_ARGUMENT;
    if (g->ny > 65535 || g->nz > 65535 || g->n_angles > 65535) return NR_ERR_BAD_GEOMETRY;
    if (!bp_tables_fit(*g)) return NR_ERR_BAD_GEOMETRY;
    return NR_OK;
}

static nr_status check_ws(const nr_geom* g, const nr_ostr_params* p, void* ws, size_t bytes,
                          Layout* L) {
    nr_status st = check_params(g, p);
    if (st != NR_OK) return st;
    *L = layout(*g, *p);
    if (!ws || bytes < L->total || ((uintptr_t)ws & 255) != 0) return NR_ERR_WORKSPACE;
    return NR_OK;
}

// Subset-major view order, Tomo_OSTR_gold.cpp:628-642: position i*Vs + j
// holds original view j*M + i.
__global__ void index_kernel(int32_t* idx, const float* __restrict__ angles_in,
                             float* __restrict__ angles_out, int A, int M) {
    const int Vs = A / M;
    for (int p = threadIdx.x; p < A; p += blockDim.x) {
        idx[p] = (p % Vs) * M + p / Vs;
        angles_out[p] = angles_in[p];
    }
}

__global__ void clear_status_kernel(int* s) {
    if (threadIdx.x < 64) s[threadIdx.x] = 0;
}

__global__ void set_word_kernel(int* p, int v) { *p = v; }

// The two set-up launches the OS-SART driver (sart.cu) shares.
nr_status launch_subset_index(int32_t* idx, const float* angles_in, float* angles_out, int A,
                              int M, cudaStream_t s) {
    index_kernel<<<1, 256, 0, s>>>(idx, angles_in, angles_out, A, M);
    return launch_status();
}

nr_status launch_clear_status(int* status, cudaStream_t s) {
    clear_status_kernel<<<1, 64, 0, s>>>(status);
    return launch_status();
}

// Section pointers of a set-up workspace, for the batched path (batch.cu).
nr_status ostr_sections(const nr_geom* g, const nr_ostr_params* p, void* ws, size_t bytes,
                        float** xtmp, float** h, const float** d, const float** y,
                        const float** b, const float** r, const float** angles,
                        const int32_t** index, int** status, BpTab* tab) {
    Layout L;
    nr_status st = check_ws(g, p, ws, bytes, &L);
    if (st != NR_OK) return st;
    WS w = carve(ws, L);
    *xtmp = w.xtmp;
    *h = w.h;
    *d = w.d;
    *y = w.y;
    *b = w.b;
    *r = w.r;
    *angles = w.angles;
    *index = w.index;
    *status = w.status;
    *tab = w.tab();
    return NR_OK;
}

}  // namespace nr

using namespace nr;

NR_API nr_status nr_validate_geometry(const nr_geom* g, int32_t subset_num) {
    if (!geom_ok(g)) return NR_ERR_BAD_GEOMETRY;
    if (g->vx != g->vy) return NR_ERR_BAD_GEOMETRY;
    if (subset_num > 0 && g->n_angles % subset_num != 0) return NR_ERR_BAD_GEOMETRY;
    return NR_OK;
}

NR_API nr_status nr_ostr_workspace_size(const nr_geom* g, const nr_ostr_params* p,
                                        size_t* bytes) {
    nr_status st = check_params(g, p);
    if (st != NR_OK) return st;
    if (!bytes) return NR_ERR_BAD_ARGUMENT;
    *bytes = layout(*g, *p).total;
    return NR_OK;
}

NR_API nr_status nr_ostr_setup(const nr_geom* g, const nr_ostr_params* p, const float* angles,
                               const float* prj, const float* blank, const float* scat,
                               void* workspace, size_t ws_bytes, void* stream) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!angles || !prj || !blank || (p->has_scatter && !scat)) return NR_ERR_BAD_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    WS w = carve(workspace, L);
    const int A = g->n_angles, M = p->subset_num, Vs = A / M;
    const int64_t N = (int64_t)g->nx * g->ny * g->nz;
    clear_status_kernel<<<1, 64, 0, s>>>(w.status);
    index_kernel<<<1, 256, 0, s>>>(w.index, angles, w.angles, A, M);
    if ((st = launch_status()) != NR_OK) return st;
    if ((st = launch_bp_tables(*g, w.angles, w.index, w.bpx, w.bpy, s)) != NR_OK) return st;
    // [view][i][j] original order -> [view][j][i] subset order.
    if ((st = launch_transpose(w.y, prj, g->nbx, g->nby, A, M, Vs, s)) != NR_OK) return st;
    if ((st = launch_transpose(w.b, blank, g->nbx, g->nby, A, M, Vs, s)) != NR_OK) return st;
    if (w.r && (st = launch_transpose(w.r, scat, g->nbx, g->nby, A, M, Vs, s)) != NR_OK) return st;
    // gamma*yry is formed in original view order (identity index, as the
    // reference does before it regroups): stage y (and r) there.
    if ((st = launch_transpose(w.gc, prj, g->nbx, g->nby, A, 0, 1, s)) != NR_OK) return st;
    if (w.r && (st = launch_transpose(w.gr, scat, g->nbx, g->nby, A, 0, 1, s)) != NR_OK) return st;
    // gc <- yry(gc, r) * gamma, original order, identity index.
    if ((st = launch_gamma_yry(*g, p->gamma_mode, w.gc, angles, w.gc, w.gr, s)) != NR_OK)
        return st;
    if (cudaMemsetAsync(w.h + (int64_t)Vs * g->nbx * g->nby, 0, bp_pad(*g) * sizeof(float), s) !=
        cudaSuccess)
        return NR_ERR_CUDA;
    if (cudaMemsetAsync(w.d, 0, N * sizeof(float), s) != cudaSuccess) return NR_ERR_CUDA;
    // d = SBP(gamma*yry) over all views, original order (Tomo_OSTR_gold.cpp:528-565).
    if ((st = launch_bp(*g, true, w.d, w.gc, angles, nullptr, 0, A, s)) != NR_OK) return st;
    return NR_OK;
}

NR_API nr_status nr_ostr_project(const nr_geom* g, const nr_ostr_params* p, const float* x,
                                 int32_t subset, void* workspace, size_t ws_bytes, void* stream) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || subset < 0 || subset >= p->subset_num) return NR_ERR_BAD_ARGUMENT;
    WS w = carve(workspace, L);
    const int Vs = g->n_angles / p->subset_num;
    return launch_fp_h(*g, p->fp_batch, p->fp_stage, x, w.h, w.angles, w.index, subset * Vs, Vs, w.y, w.b, w.r, w.status, nullptr,
                       as_stream(stream));
}

NR_API nr_status nr_ostr_update(const nr_geom* g, const nr_ostr_params* p, const float* x,
                                float* x_out, int32_t subset, void* workspace, size_t ws_bytes,
                                void* stream) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || !x_out || x == x_out || subset < 0 || subset >= p->subset_num)
        return NR_ERR_BAD_ARGUMENT;
    WS w = carve(workspace, L);
    const int M = p->subset_num, Vs = g->n_angles / M;
    CUtensorMap map;
    const bool mapped = update_map(*g, *p, x, &map);
    return launch_update(*g, p->potential, p->upd_planes, p->upd_tile, x, x_out, w.d, w.h,
                         w.angles, w.index, w.tab(), subset * Vs, Vs, (float)M, p->beta, p->delta,
                         w.status, mapped ? &map : nullptr, as_stream(stream));
}

NR_API nr_status nr_ostr_workspace_section(const nr_geom* g, const nr_ostr_params* p,
                                           int32_t section, void* workspace, size_t ws_bytes,
                                           void** ptr, size_t* bytes) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!ptr || !bytes) return NR_ERR_BAD_ARGUMENT;
    WS w = carve(workspace, L);
    const int64_t A = g->n_angles, B = (int64_t)g->nbx * g->nby;
    const int64_t N = (int64_t)g->nx * g->ny * g->nz;
    switch (section) {
    case NR_WS_D: *ptr = w.d; *bytes = N * sizeof(float); break;
    case NR_WS_H: *ptr = w.h; *bytes = (A / p->subset_num) * B * sizeof(float); break;
    case NR_WS_Y: *ptr = w.y; *bytes = A * B * sizeof(float); break;
    case NR_WS_GAMMA_YRY: *ptr = w.gc; *bytes = A * B * sizeof(float); break;
    case NR_WS_INDEX: *ptr = w.index; *bytes = A * sizeof(int32_t); break;
    default: return NR_ERR_BAD_ARGUMENT;
    }
    return NR_OK;
}

NR_API nr_status nr_ostr_subiter(const nr_geom* g, const nr_ostr_params* p, float* x,
                                 int32_t subset, void* workspace, size_t ws_bytes, void* stream) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || subset < 0 || subset >= p->subset_num) return NR_ERR_BAD_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    WS w = carve(workspace, L);
    const int A = g->n_angles, M = p->subset_num, Vs = A / M;
    const int64_t N = (int64_t)g->nx * g->ny * g->nz;
    const int a0 = subset * Vs;
    if ((st = launch_fp_h(*g, p->fp_batch, p->fp_stage, x, w.h, w.angles, w.index, a0, Vs, w.y, w.b, w.r, w.status, nullptr, s)) != NR_OK)
        return st;
    CUtensorMap map;
    const bool mapped = update_map(*g, *p, x, &map);
    if ((st = launch_update(*g, p->potential, p->upd_planes, p->upd_tile, x, w.xtmp, w.d, w.h,
                            w.angles, w.index, w.tab(), a0, Vs, (float)M, p->beta, p->delta,
                            w.status, mapped ? &map : nullptr, s)) != NR_OK)
        return st;
    if (cudaMemcpyAsync(x, w.xtmp, N * sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return NR_ERR_CUDA;
    return NR_OK;
}

// Enqueues n_iters iterations on stream s (ping-pong between x and xtmp).
static nr_status enqueue_iterations(const nr_geom* g, const nr_ostr_params* p, float* x,
                                    int32_t n_iters, const WS& w, cudaStream_t s) {
    const int A = g->n_angles, M = p->subset_num, Vs = A / M;
    const int64_t N = (int64_t)g->nx * g->ny * g->nz;
    nr_status st;
    float* cur = x;
    float* nxt = w.xtmp;
    // the staged projection's descriptors of the two volume buffers, once
    CUtensorMap maps[2];
    const bool staged = p->fp_stage == NR_STAGE_TMA && p->fp_batch != 8 &&
                        slab_map(*g, x, &maps[0]) && slab_map(*g, w.xtmp, &maps[1]);
    // and the TMA-fed update's
    CUtensorMap umaps[2];
    const bool umapped = update_map(*g, *p, x, &umaps[0]) && update_map(*g, *p, w.xtmp, &umaps[1]);
    for (int it = 0; it < n_iters; it++) {
        for (int a = 0; a < M; a++) {
            const int a0 = a * Vs;
            if ((st = launch_fp_h(*g, p->fp_batch, p->fp_stage, cur, w.h, w.angles, w.index, a0, Vs, w.y, w.b, w.r, w.status,
                                  staged ? &maps[cur == x ? 0 : 1] : nullptr, s)) !=
                NR_OK)
                return st;
            if ((st = launch_update(*g, p->potential, p->upd_planes, p->upd_tile, cur, nxt, w.d,
                                    w.h, w.angles, w.index, w.tab(), a0, Vs, (float)M, p->beta,
                                    p->delta, w.status,
                                    umapped ? &umaps[cur == x ? 0 : 1] : nullptr, s)) != NR_OK)
                return st;
            float* t = cur;
            cur = nxt;
            nxt = t;
        }
    }
    if (cur != x &&
        cudaMemcpyAsync(x, cur, N * sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return NR_ERR_CUDA;
    return NR_OK;
}

NR_API nr_status nr_ostr_iterate(const nr_geom* g, const nr_ostr_params* p, float* x,
                                 int32_t n_iters, void* workspace, size_t ws_bytes, void* stream) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || n_iters < 0) return NR_ERR_BAD_ARGUMENT;
    return enqueue_iterations(g, p, x, n_iters, carve(workspace, L), as_stream(stream));
}

NR_API nr_status nr_ostr_graph_create(const nr_geom* g, const nr_ostr_params* p, float* x,
                                      int32_t n_iters, void* workspace, size_t ws_bytes,
                                      void* stream, void** graph) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || n_iters < 1 || !graph || !stream) return NR_ERR_BAD_ARGUMENT;
    *graph = nullptr;
    cudaStream_t s = as_stream(stream);
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return NR_ERR_CUDA;
    st = enqueue_iterations(g, p, x, n_iters, carve(workspace, L), s);
    return finish_capture(s, st, graph);
}

NR_API nr_status nr_ostr_graph_launch(void* graph, void* stream) {
    if (!graph) return NR_ERR_BAD_ARGUMENT;
    auto* h = static_cast<GraphHandle*>(graph);
    return cudaGraphLaunch(h->exec, as_stream(stream)) == cudaSuccess ? NR_OK : NR_ERR_CUDA;
}

NR_API nr_status nr_ostr_graph_destroy(void* graph) {
    if (!graph) return NR_OK;
    auto* h = static_cast<GraphHandle*>(graph);
    cudaGraphExecDestroy(h->exec);
    cudaGraphDestroy(h->graph);
    delete h;
    return NR_OK;
}

NR_API nr_status nr_ostr_objective(const nr_geom* g, const nr_ostr_params* p, const float* x,
                                   double* out, void* workspace, size_t ws_bytes, void* stream) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || !out) return NR_ERR_BAD_ARGUMENT;
    WS w = carve(workspace, L);
    return launch_objective(*g, p->potential, p->delta, x, w.angles, w.index, w.y, w.b, w.r, w.red,
                            w.red_n, out, as_stream(stream));
}

NR_API nr_status nr_ostr_project_fp64(const nr_geom* g, const nr_ostr_params* p, const float* x,
                                      int32_t subset, double* data_out, void* workspace,
                                      size_t ws_bytes, void* stream) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || !data_out || subset < 0 || subset >= p->subset_num) return NR_ERR_BAD_ARGUMENT;
    WS w = carve(workspace, L);
    const int Vs = g->n_angles / p->subset_num;
    return launch_fp_h_data(*g, p->fp_batch, x, w.h, w.angles, w.index, subset * Vs, Vs, w.y,
                            w.b, w.r, w.red, w.red_n, data_out, as_stream(stream));
}

NR_API nr_status nr_ostr_penalty(const nr_geom* g, const nr_ostr_params* p, const float* x,
                                 double* out, void* workspace, size_t ws_bytes, void* stream) {
    Layout L;
    nr_status st = check_ws(g, p, workspace, ws_bytes, &L);
    if (st != NR_OK) return st;
    if (!x || !out) return NR_ERR_BAD_ARGUMENT;
    WS w = carve(workspace, L);
    return launch_penalty(*g, p->potential, p->delta, x, w.red, w.red_n, out, as_stream(stream));
}

NR_API nr_status nr_ostr_check(void* workspace, size_t ws_bytes, int32_t* flags, void* stream) {
    if (!workspace || ws_bytes < 256 || !flags) return NR_ERR_BAD_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    int v = 0;
    if (cudaMemcpyAsync(&v, workspace, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return NR_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return NR_ERR_CUDA;
    *flags = v;
    if (v) {
        clear_status_kernel<<<1, 64, 0, s>>>((int*)workspace);
        if (launch_status() != NR_OK) return NR_ERR_LAUNCH;
    }
    if (v & NR_FLAG_TIMEOUT) return NR_ERR_TIMEOUT;
    if (v & NR_FLAG_NONFINITE) return NR_ERR_NONFINITE;
    return NR_OK;
}

NR_API nr_status nr_test_expire_wait(void* workspace, int32_t wait_index, void* stream) {
    if (!workspace || ((uintptr_t)workspace & 255) != 0) return NR_ERR_BAD_ARGUMENT;
    set_word_kernel<<<1, 1, 0, as_stream(stream)>>>((int*)workspace + 1,
                                                   wait_index < 0 ? 0 : wait_index + 1);
    return launch_status();
}

NR_API const char* nr_version(void) { return "nrgb300 0.1.0 sm_103a"; }

NR_API nr_status nr_ostr_subset(const nr_geom* g, const nr_ostr_params* p, float* x,
                                int32_t subset, void* workspace, size_t ws_bytes, void* stream) {
    return nr_ostr_subiter(g, p, x, subset, workspace, ws_bytes, stream);
}

NR_API nr_status nr_objective_fp64(const nr_geom* g, const nr_ostr_params* p, const float* x,
                                   double* out, void* workspace, size_t ws_bytes, void* stream) {
    return nr_ostr_objective(g, p, x, out, workspace, ws_bytes, stream);
}

NR_API nr_status nr_workspace_size(const nr_geom* g, const nr_ostr_params* p, size_t* bytes) {
    return nr_ostr_workspace_size(g, p, bytes);
}
