// batch.cu -- many independent reconstructions advanced by shared launches.
//
// A batch step advances every unfinished case by one sub-iteration: one
// launch of the fused forward projection + gradient of all cases, then one
// update launch per (potential, update form, slab depth) class.  Each launch
// walks one flat list of work items -- (case, detector tile, view) or (case,
// volume tile, z chunk) -- built from per-case prefix offsets, so cases of
// different sizes, view counts and potentials share the GPU in the same launch
// and small cases fill the SMs that large ones leave idle.  Case c works on
// subset (step mod M_c) and ping-pongs x <-> xtmp; it stops after
// n_iters_c * M_c steps, and nr_batch_finish moves an odd-parity result back
// into x.  The tile bodies are the single-case ones (project.cuh, update.cuh),
// so a batched case computes exactly what nr_ostr_iterate does.
//
// Scheduling: one block per work item, so the hardware block scheduler is the
// work queue and uneven tiles balance themselves.  (A persistent grid of
// SMs x resident blocks with a static grid-stride split of the same items
// measured 12-21 % slower than the cases run one after another, because the
// static split leaves SMs idle behind blocks that drew expensive tiles.)  Cases
// are ordered by sub-iteration count, longest first, within each class and
// in the projection order, so the cases still running at step k are a prefix
// of every item range and each launch covers exactly the active items.
//
// The case table travels as a __grid_constant__ kernel parameter (at most
// 64 cases: ~19 KB, inside the 32 KB parameter limit).  The item decode then
// runs on block-uniform constant-bank values and the tile reads its case's
// geometry from the constant bank as the single-case kernels do, instead of
// from a shared-memory copy that costs registers: the one-voxel one-view
// update fits 32 registers (8 resident blocks per SM; 8 bytes spill).
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "project.cuh"
#include "update.cuh"

namespace nr {

constexpr int BATCH_MAX = 64;
constexpr int N_ZC = 3;                      // update slab depths 8, 16, 32 planes
// update forms: several views per subset; one view, one voxel per thread;
// one view, two voxels per thread (the case's upd_tile)
constexpr int N_FORM = 3;
constexpr int N_CLASSES = 4 * N_FORM * N_ZC; // potential x form x slab depth

struct CaseDev {
    Geo G;
    PriorW5 W;
    float beta, delta, M;
    int pot, Vs, total_sub;
    float* x;
    float* xtmp;
    float* h;
    const float *d, *y, *b, *r, *angles;
    const int32_t* index;
    int* status;
    BpTab T;               // the case's back-projection tables
    int fp_tx, fp_ty;      // detector tiles of 32 x 4 bins
    int up_tx, up_ty;      // volume tiles of 32 x 8 columns (64 x 8 in form 2)
    int form;              // update form (N_FORM)
    int zc;                // z planes per update item (the plan's upd_planes)
    int64_t N;
};

__host__ __device__ constexpr int zc_index(int zc) { return zc == 8 ? 0 : (zc == 32 ? 2 : 1); }
__host__ __device__ constexpr int upd_form(bool one_view, int tile) {
    return one_view ? (tile == NR_TILE_2 ? 2 : 1) : 0;
}
__host__ __device__ constexpr int upd_class(int pot, int form, int zc) {
    return (N_FORM * pot + form) * N_ZC + zc_index(zc);
}

struct BatchTable {
    int n;
    // cases c[] are in class order (potential, update form, slab depth), and
    // by sub-iteration count, longest first, within a class
    int cls_first[N_CLASSES], cls_end[N_CLASSES];  // cases [first, end) of each class
    int up_off[BATCH_MAX + 1];                     // update items: prefix over c[]
    int fp_case[BATCH_MAX];                        // projection order (longest first)
    int fp_off[BATCH_MAX + 1];                     // projection items: prefix over fp_case
    CaseDev c[BATCH_MAX];
};
static_assert(sizeof(BatchTable) <= 32764 - 16, "kernel parameter limit");

__device__ __forceinline__ int find_case(const int* off, int n, int it) {
    int c = 0;
    while (c + 1 < n && it >= off[c + 1]) c++;
    return c;
}

// Projection items [0, hi) of step `step` (hi: the active prefix).  12 resident
// blocks per SM, as fp_h_kernel.
__global__ void __launch_bounds__(128, 12) fp_batch_kernel(const __grid_constant__ BatchTable P,
                                                           int step, int hi) {
    __shared__ ViewSrc src;
    for (int it = blockIdx.x; it < hi; it += gridDim.x) {
        const int p = find_case(P.fp_off, P.n, it);
        const CaseDev& cd = P.c[P.fp_case[p]];
        __syncthreads();  // previous item's readers of src are done
        if (step >= cd.total_sub) continue;
        const int local = it - P.fp_off[p];
        const int bx = local % cd.fp_tx;
        const int by = (local / cd.fp_tx) % cd.fp_ty;
        const int bz = local / (cd.fp_tx * cd.fp_ty);
        const int a0 = (step % (int)cd.M) * cd.Vs;
        const float* cur = (step & 1) ? cd.xtmp : cd.x;
        const Geo G = cd.G;  // copied once per item, as in update_batch_kernel
        fp_h_tile(G, cur, cd.h, cd.angles, cd.index, a0, cd.y, cd.b, cd.r, bx, by, bz, src);
    }
}

// Update items [lo, hi) of one (potential, NV, ZC, X2) class.  NV = 1 serves
// the cases whose subsets hold one view (the compile-time view count of
// update_tile: 32 registers, 8 resident blocks per SM); NV = 0 the others
// (no block minimum, as update_kernel: 40 registers).  X2: the one-view
// cases that take two voxels per thread (update_tile_x2, 5 blocks per SM as
// update_x2_kernel).  ZC is the case's slab depth (planes per item), as the
// autotuner picked it.
template <int POT, int NV, int ZC, bool X2>
__global__ void __launch_bounds__(256, NV ? (X2 ? 5 : 8) : 0) update_batch_kernel(
    const __grid_constant__ BatchTable P, int step, int lo, int hi) {
    __shared__ typename std::conditional<X2, UpdSmem2, UpdSmem>::type sm;
    for (int it = lo + blockIdx.x; it < hi; it += gridDim.x) {
        const int c = find_case(P.up_off, P.n, it);
        const CaseDev& cd = P.c[c];
        __syncthreads();  // previous item's readers of sm are done
        if (step >= cd.total_sub) continue;
        const int local = it - P.up_off[c];
        const int bx = local % cd.up_tx;
        const int by = (local / cd.up_tx) % cd.up_ty;
        const int bz = local / (cd.up_tx * cd.up_ty);
        const int a0 = (step % (int)cd.M) * cd.Vs;
        const float* cur = (step & 1) ? cd.xtmp : cd.x;
        float* nxt = (step & 1) ? cd.x : cd.xtmp;
        // The tile reads its case's values from locals copied once per item:
        // read through the runtime case index, they were fetched again on
        // every plane (8 % more instructions than the single-case kernel,
        // whose fixed constant-bank offsets are free operands).
        const Geo G = cd.G;
        const PriorW5 W = cd.W;
        const BpTab T = cd.T;
        if constexpr (X2)
            update_tile_x2<POT, ZC, UPD_OSTR, NV>(G, W, cur, nxt, cd.d, cd.h, cd.angles, cd.index,
                                                  T, a0, cd.Vs, cd.M, cd.beta, cd.delta,
                                                  cd.status, bx, by, bz, sm);
        else
            update_tile<POT, ZC, UPD_OSTR, NV>(G, W, cur, nxt, cd.d, cd.h, cd.angles, cd.index, T,
                                                a0, cd.Vs, cd.M, cd.beta, cd.delta, cd.status, bx,
                                                by, bz, sm);
    }
}

// Cases whose sub-iteration count is odd end in xtmp: copy them back to x.
__global__ void finish_kernel(const __grid_constant__ BatchTable P) {
    for (int c = 0; c < P.n; c++) {
        if ((P.c[c].total_sub & 1) == 0) continue;
        const float* __restrict__ s = P.c[c].xtmp;
        float* __restrict__ dst = P.c[c].x;
        for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < P.c[c].N;
             k += (int64_t)gridDim.x * blockDim.x)
            dst[k] = s[k];
    }
}

// Workspace section pointers of one case (the layout of ostr.cu).
nr_status ostr_sections(const nr_geom* g, const nr_ostr_params* p, void* ws, size_t bytes,
                        float** xtmp, float** h, const float** d, const float** y,
                        const float** b, const float** r, const float** angles,
                        const int32_t** index, int** status, BpTab* tab);

// A table written by nr_batch_prepare: its counts and offsets are consistent
// (a table from anywhere else is refused).
static bool table_ok(const void* table) {
    if (!table || ((uintptr_t)table & 7) != 0) return false;
    const BatchTable& P = *(const BatchTable*)table;
    if (P.n < 1 || P.n > BATCH_MAX || P.fp_off[0] != 0 || P.up_off[0] != 0) return false;
    bool seen[BATCH_MAX] = {};
    for (int c = 0; c < P.n; c++) {
        if (P.fp_off[c + 1] < P.fp_off[c] || P.up_off[c + 1] < P.up_off[c]) return false;
        const int f = P.fp_case[c];
        if (f < 0 || f >= P.n || seen[f]) return false;
        seen[f] = true;
    }
    for (int k = 0; k < N_CLASSES; k++)
        if (P.cls_first[k] < 0 || P.cls_first[k] > P.cls_end[k] || P.cls_end[k] > P.n)
            return false;
    return true;
}

}  // namespace nr

using namespace nr;

NR_API nr_status nr_batch_table_size(int32_t n_cases, size_t* bytes) {
    if (n_cases <= 0 || n_cases > BATCH_MAX || !bytes) return NR_ERR_BAD_ARGUMENT;
    *bytes = sizeof(BatchTable);
    return NR_OK;
}

NR_API nr_status nr_batch_prepare(const nr_batch_case* cases, int32_t n_cases, void* table,
                                  size_t table_bytes, int32_t* n_steps, void* stream) {
    (void)stream;
    size_t need = 0;
    nr_status st = nr_batch_table_size(n_cases, &need);
    if (st != NR_OK) return st;
    if (!cases || !table || table_bytes < need || ((uintptr_t)table & 7) != 0)
        return NR_ERR_WORKSPACE;
    for (int c = 0; c < n_cases; c++) {
        const nr_batch_case& k = cases[c];
        if (k.n_iters < 0 || !k.x || k.p.subset_num < 1 || k.p.potential < NR_POT_Q2 ||
            k.p.potential > NR_POT_HUBER ||
            (k.p.upd_planes != 0 && k.p.upd_planes != 8 && k.p.upd_planes != 16 &&
             k.p.upd_planes != 32) ||
            (k.p.upd_tile != NR_TILE_1 && k.p.upd_tile != NR_TILE_2 &&
             k.p.upd_tile != NR_TILE_TMA))
            return NR_ERR_BAD_ARGUMENT;
    }
    auto total_sub = [&](int c) { return cases[c].n_iters * cases[c].p.subset_num; };
    auto zc_of = [&](int c) { return cases[c].p.upd_planes == 0 ? UZC : cases[c].p.upd_planes; };
    auto cls_of = [&](int c) {
        const nr_batch_case& k = cases[c];
        return upd_class(k.p.potential, upd_form(k.g.n_angles == k.p.subset_num, k.p.upd_tile),
                         zc_of(c));
    };
    // case order: by class, then by sub-iteration count, longest first (stable)
    int order[BATCH_MAX];
    for (int c = 0; c < n_cases; c++) order[c] = c;
    for (int i = 1; i < n_cases; i++) {
        const int v = order[i];
        int j = i;
        while (j > 0 && (cls_of(order[j - 1]) > cls_of(v) ||
                         (cls_of(order[j - 1]) == cls_of(v) && total_sub(order[j - 1]) < total_sub(v)))) {
            order[j] = order[j - 1];
            j--;
        }
        order[j] = v;
    }
    BatchTable* P = new BatchTable();
    P->n = n_cases;
    int steps = 0;
    int64_t up_off = 0;
    for (int c = 0; c < n_cases; c++) {
        const nr_batch_case& k = cases[order[c]];
        CaseDev& d = P->c[c];
        st = ostr_sections(&k.g, &k.p, k.workspace, k.ws_bytes, &d.xtmp, &d.h, &d.d, &d.y, &d.b,
                           &d.r, &d.angles, &d.index, &d.status, &d.T);
        if (st != NR_OK) {
            delete P;
            return st;
        }
        const nr_geom& g = k.g;
        d.G = make_geo(g);
        d.W = make_w5(g.vz / g.vx, k.p.delta);
        d.beta = k.p.beta;
        d.delta = k.p.potential == NR_POT_Q2 ? 1.f : k.p.delta;
        d.M = (float)k.p.subset_num;
        d.pot = k.p.potential;
        d.Vs = g.n_angles / k.p.subset_num;
        d.total_sub = total_sub(order[c]);
        d.x = k.x;
        d.fp_tx = (int)cdiv(g.nbx, 32);
        d.fp_ty = (int)cdiv(g.nby, 4);
        d.form = upd_form(d.Vs == 1, k.p.upd_tile);
        d.up_tx = (int)cdiv(g.nx, d.form == 2 ? U2X : UTX);
        d.up_ty = (int)cdiv(g.ny, UTY);
        d.zc = zc_of(order[c]);
        d.N = (int64_t)g.nx * g.ny * g.nz;
        up_off += (int64_t)d.up_tx * d.up_ty * cdiv(g.nz, d.zc);
        if (up_off > INT32_MAX) {
            delete P;
            return NR_ERR_BAD_ARGUMENT;  // work items are counted in 32 bits
        }
        P->up_off[c + 1] = (int)up_off;
        steps = d.total_sub > steps ? d.total_sub : steps;
    }
    for (int k = 0; k < N_CLASSES; k++) P->cls_first[k] = P->cls_end[k] = 0;
    for (int c = n_cases - 1; c >= 0; c--) {
        const int k = upd_class(P->c[c].pot, P->c[c].form, P->c[c].zc);
        if (P->cls_end[k] == 0) P->cls_end[k] = c + 1;
        P->cls_first[k] = c;
    }
    // projection order: all cases by sub-iteration count, longest first (stable)
    for (int c = 0; c < n_cases; c++) P->fp_case[c] = c;
    for (int i = 1; i < n_cases; i++) {
        const int v = P->fp_case[i];
        int j = i;
        while (j > 0 && P->c[P->fp_case[j - 1]].total_sub < P->c[v].total_sub) {
            P->fp_case[j] = P->fp_case[j - 1];
            j--;
        }
        P->fp_case[j] = v;
    }
    int64_t fp_off = 0;
    for (int p = 0; p < n_cases; p++) {
        const CaseDev& d = P->c[P->fp_case[p]];
        fp_off += (int64_t)d.fp_tx * d.fp_ty * d.Vs;
        if (fp_off > INT32_MAX) {
            delete P;
            return NR_ERR_BAD_ARGUMENT;
        }
        P->fp_off[p + 1] = (int)fp_off;
    }
    memcpy(table, P, sizeof(BatchTable));
    delete P;
    if (n_steps) *n_steps = steps;
    return NR_OK;
}

namespace {

template <int POT, int NV, int ZC, bool X2>
void launch_class_t(const BatchTable& P, int32_t k, int lo, int hi, cudaStream_t s) {
    update_batch_kernel<POT, NV, ZC, X2><<<hi - lo, dim3(UTX, UTY), 0, s>>>(P, k, lo, hi);
}

template <int POT, int NV, bool X2>
void launch_class_z(int zi, const BatchTable& P, int32_t k, int lo, int hi, cudaStream_t s) {
    if (zi == 0) return launch_class_t<POT, NV, 8, X2>(P, k, lo, hi, s);
    if (zi == 2) return launch_class_t<POT, NV, 32, X2>(P, k, lo, hi, s);
    return launch_class_t<POT, NV, 16, X2>(P, k, lo, hi, s);
}

template <int POT>
void launch_class_form(int form, int zi, const BatchTable& P, int32_t k, int lo, int hi,
                       cudaStream_t s) {
    if (form == 2) return launch_class_z<POT, 1, true>(zi, P, k, lo, hi, s);
    if (form == 1) return launch_class_z<POT, 1, false>(zi, P, k, lo, hi, s);
    return launch_class_z<POT, 0, false>(zi, P, k, lo, hi, s);
}

void launch_class(int cls, const BatchTable& P, int32_t k, int lo, int hi, cudaStream_t s) {
    const int zi = cls % N_ZC, form = (cls / N_ZC) % N_FORM, pot = cls / (N_FORM * N_ZC);
    switch (pot) {
    case NR_POT_Q2: return launch_class_form<NR_POT_Q2>(form, zi, P, k, lo, hi, s);
    case NR_POT_LANGE: return launch_class_form<NR_POT_LANGE>(form, zi, P, k, lo, hi, s);
    case NR_POT_HYPERBOLA: return launch_class_form<NR_POT_HYPERBOLA>(form, zi, P, k, lo, hi, s);
    default: return launch_class_form<NR_POT_HUBER>(form, zi, P, k, lo, hi, s);
    }
}

// Steps first .. first+count-1: the projection of the active items, then one
// update launch per class that has active cases (one block per item; the
// active cases are a prefix of each range, so finished cases cost nothing).
nr_status enqueue_steps(const BatchTable& P, int32_t first, int32_t count, cudaStream_t s) {
    for (int32_t k = first; k < first + count; k++) {
        int np = 0;
        while (np < P.n && P.c[P.fp_case[np]].total_sub > k) np++;
        if (np == 0) continue;  // every case is done
        fp_batch_kernel<<<P.fp_off[np], dim3(32, 4), 0, s>>>(P, k, P.fp_off[np]);
        for (int cls = 0; cls < N_CLASSES; cls++) {
            int e = P.cls_first[cls];
            while (e < P.cls_end[cls] && P.c[e].total_sub > k) e++;
            const int lo = P.up_off[P.cls_first[cls]], hi = P.up_off[e];
            if (hi > lo) launch_class(cls, P, k, lo, hi, s);
        }
    }
    return launch_status();
}

}  // namespace

NR_API nr_status nr_batch_step(const void* table, int32_t step, void* stream) {
    if (!table_ok(table) || step < 0) return NR_ERR_BAD_ARGUMENT;
    return enqueue_steps(*(const BatchTable*)table, step, 1, as_stream(stream));
}

NR_API nr_status nr_batch_finish(const void* table, void* stream) {
    if (!table_ok(table)) return NR_ERR_BAD_ARGUMENT;
    finish_kernel<<<1024, 256, 0, as_stream(stream)>>>(*(const BatchTable*)table);
    return launch_status();
}

NR_API nr_status nr_batch_graph_create(const void* table, int32_t n_steps, void* stream,
                                       void** graph) {
    if (!table_ok(table) || n_steps < 1 || !graph || !stream) return NR_ERR_BAD_ARGUMENT;
    *graph = nullptr;
    const BatchTable& P = *(const BatchTable*)table;
    cudaStream_t s = as_stream(stream);
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return NR_ERR_CUDA;
    nr_status st = enqueue_steps(P, 0, n_steps, s);
    if (st == NR_OK) {
        finish_kernel<<<1024, 256, 0, s>>>(P);
        st = launch_status();
    }
    return finish_capture(s, st, graph);
}
