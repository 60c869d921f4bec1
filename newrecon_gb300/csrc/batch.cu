// batch.cu -- many independent reconstructions in one persistent launch.
//
// A batch step advances every unfinished case by one sub-iteration with two
// persistent launches (grid = SMs x resident blocks): the fused forward
// projection + gradient of all cases, then the fused update of all cases.
// Each launch walks one flat list of work items -- (case, detector tile, view)
// or (case, volume tile, z chunk) -- built from per-case prefix offsets, so
// cases of different sizes, view counts and potentials share the GPU in the
// same launch and small cases fill the SMs that large ones leave idle.
// Case c works on subset (step mod M_c) and ping-pongs x <-> xtmp; it stops
// after n_iters_c * M_c steps, and nr_batch_finish moves an odd-parity result
// back into x.  The tile bodies are the single-case ones (project.cuh,
// update.cuh), so a batched case computes exactly what nr_ostr_iterate does.
#include "project.cuh"
#include "update.cuh"

namespace nr {

constexpr int BATCH_MAX = 64;

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
    int up_tx, up_ty;      // volume tiles of 32 x 8 columns (z chunks of UZC planes)
    int64_t N;
};

struct BatchHdr {
    int n;
    int64_t fp_total, up_total;
    int64_t fp_off[BATCH_MAX + 1], up_off[BATCH_MAX + 1];
    int64_t pot_lo[4], pot_hi[4];  // update items of each potential (cases sorted by potential)
};

constexpr size_t HDR_BYTES = (sizeof(BatchHdr) + 255) & ~(size_t)255;

__device__ __forceinline__ int find_case(const int64_t* off, int n, int64_t it) {
    int c = 0;
    while (c + 1 < n && it >= off[c + 1]) c++;
    return c;
}

// All threads copy case c's descriptor into shared memory (word by word).
__device__ __forceinline__ void load_case(CaseDev& dst, const CaseDev* C, int c, int tid,
                                          int nthreads) {
    static_assert(sizeof(CaseDev) % 4 == 0, "word copy");
    const int* src = (const int*)(C + c);
    int* d = (int*)&dst;
    for (int k = tid; k < (int)(sizeof(CaseDev) / 4); k += nthreads) d[k] = src[k];
}

__global__ void __launch_bounds__(128) fp_batch_kernel(const void* __restrict__ table, int step) {
    __shared__ CaseDev cd;
    __shared__ ViewSrc src;
    const BatchHdr* H = (const BatchHdr*)table;
    const CaseDev* C = (const CaseDev*)((const char*)table + HDR_BYTES);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int64_t it = blockIdx.x; it < H->fp_total; it += gridDim.x) {
        const int c = find_case(H->fp_off, H->n, it);
        __syncthreads();  // previous item's readers of cd / src are done
        load_case(cd, C, c, tid, 128);
        __syncthreads();
        if (step >= cd.total_sub) continue;
        const int64_t local = it - H->fp_off[c];
        const int bx = (int)(local % cd.fp_tx);
        const int by = (int)((local / cd.fp_tx) % cd.fp_ty);
        const int bz = (int)(local / ((int64_t)cd.fp_tx * cd.fp_ty));
        const int a0 = (step % (int)cd.M) * cd.Vs;
        const float* cur = (step & 1) ? cd.xtmp : cd.x;
        fp_h_tile(cd.G, cur, cd.h, cd.angles, cd.index, a0, cd.y, cd.b, cd.r, bx, by, bz, src);
    }
}

template <int POT>
__global__ void __launch_bounds__(256, 5) update_batch_kernel(const void* __restrict__ table,
                                                           int step) {
    __shared__ CaseDev cd;
    __shared__ UpdSmem sm;
    const BatchHdr* H = (const BatchHdr*)table;
    const CaseDev* C = (const CaseDev*)((const char*)table + HDR_BYTES);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int64_t it = H->pot_lo[POT] + blockIdx.x; it < H->pot_hi[POT]; it += gridDim.x) {
        const int c = find_case(H->up_off, H->n, it);
        __syncthreads();
        load_case(cd, C, c, tid, 256);
        __syncthreads();
        if (step >= cd.total_sub) continue;
        const int64_t local = it - H->up_off[c];
        const int bx = (int)(local % cd.up_tx);
        const int by = (int)((local / cd.up_tx) % cd.up_ty);
        const int bz = (int)(local / ((int64_t)cd.up_tx * cd.up_ty));
        const int a0 = (step % (int)cd.M) * cd.Vs;
        const float* cur = (step & 1) ? cd.xtmp : cd.x;
        float* nxt = (step & 1) ? cd.x : cd.xtmp;
        update_tile<POT>(cd.G, cd.W, cur, nxt, cd.d, cd.h, cd.angles, cd.index, cd.T, a0, cd.Vs, cd.M,
                         cd.beta, cd.delta, cd.status, bx, by, bz, sm);
    }
}

// Cases whose sub-iteration count is odd end in xtmp: copy them back to x.
__global__ void finish_kernel(const void* __restrict__ table) {
    const BatchHdr* H = (const BatchHdr*)table;
    const CaseDev* C = (const CaseDev*)((const char*)table + HDR_BYTES);
    for (int c = 0; c < H->n; c++) {
        if ((C[c].total_sub & 1) == 0) continue;
        const float* __restrict__ s = C[c].xtmp;
        float* __restrict__ dst = C[c].x;
        for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < C[c].N;
             k += (int64_t)gridDim.x * blockDim.x)
            dst[k] = s[k];
    }
}

// Workspace section pointers of one case (the layout of ostr.cu).
nr_status ostr_sections(const nr_geom* g, const nr_ostr_params* p, void* ws, size_t bytes,
                        float** xtmp, float** h, const float** d, const float** y,
                        const float** b, const float** r, const float** angles,
                        const int32_t** index, int** status, BpTab* tab);

static int persistent_blocks(const void* kernel, int threads, size_t smem) {
    int dev = 0, sms = 152, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
    return sms * (per > 0 ? per : 1);
}

}  // namespace nr

using namespace nr;

NR_API nr_status nr_batch_table_size(int32_t n_cases, size_t* bytes) {
    if (n_cases <= 0 || n_cases > BATCH_MAX || !bytes) return NR_ERR_BAD_ARGUMENT;
    *bytes = HDR_BYTES + (size_t)n_cases * sizeof(CaseDev);
    return NR_OK;
}

NR_API nr_status nr_batch_prepare(const nr_batch_case* cases, int32_t n_cases, void* table,
                                  size_t table_bytes, int32_t* n_steps, void* stream) {
    size_t need = 0;
    nr_status st = nr_batch_table_size(n_cases, &need);
    if (st != NR_OK) return st;
    if (!cases || !table || table_bytes < need || ((uintptr_t)table & 255) != 0)
        return NR_ERR_WORKSPACE;
    static_assert(sizeof(BatchHdr) <= HDR_BYTES, "header");
    // Host image of the table; copied to the device with one cudaMemcpyAsync.
    char* img = new char[need]();
    BatchHdr* H = (BatchHdr*)img;
    CaseDev* C = (CaseDev*)(img + HDR_BYTES);
    H->n = n_cases;
    int steps = 0;
    // cases ordered by potential, so each potential's update items are one range
    int order[BATCH_MAX];
    int no = 0;
    for (int pot = NR_POT_Q2; pot <= NR_POT_HUBER; pot++)
        for (int c = 0; c < n_cases; c++)
            if (cases[c].p.potential == pot) order[no++] = c;
    if (no != n_cases) {
        delete[] img;
        return NR_ERR_BAD_ARGUMENT;  // unknown potential
    }
    for (int c = 0; c < n_cases; c++) {
        const nr_batch_case& k = cases[order[c]];
        CaseDev& d = C[c];
        if (k.n_iters < 0 || !k.x) {
            delete[] img;
            return NR_ERR_BAD_ARGUMENT;
        }
        st = ostr_sections(&k.g, &k.p, k.workspace, k.ws_bytes, &d.xtmp, &d.h, &d.d, &d.y, &d.b,
                           &d.r, &d.angles, &d.index, &d.status, &d.T);
        if (st != NR_OK) {
            delete[] img;
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
        d.total_sub = k.n_iters * k.p.subset_num;
        d.x = k.x;
        d.fp_tx = (int)cdiv(g.nbx, 32);
        d.fp_ty = (int)cdiv(g.nby, 4);
        d.up_tx = (int)cdiv(g.nx, UTX);
        d.up_ty = (int)cdiv(g.ny, UTY);
        d.N = (int64_t)g.nx * g.ny * g.nz;
        H->fp_off[c + 1] = H->fp_off[c] + (int64_t)d.fp_tx * d.fp_ty * d.Vs;
        H->up_off[c + 1] = H->up_off[c] + (int64_t)d.up_tx * d.up_ty * cdiv(g.nz, UZC);
        steps = d.total_sub > steps ? d.total_sub : steps;
    }
    H->fp_total = H->fp_off[n_cases];
    H->up_total = H->up_off[n_cases];
    for (int pot = 0; pot < 4; pot++) {
        H->pot_lo[pot] = H->up_total;
        H->pot_hi[pot] = H->up_total;
    }
    for (int c = n_cases - 1; c >= 0; c--) {
        const int pot = C[c].pot;
        H->pot_lo[pot] = H->up_off[c];
        if (H->pot_hi[pot] == H->up_total && (c == n_cases - 1 || C[c + 1].pot != pot))
            H->pot_hi[pot] = H->up_off[c + 1];
    }
    const cudaError_t e =
        cudaMemcpyAsync(table, img, need, cudaMemcpyHostToDevice, as_stream(stream));
    const cudaError_t e2 = cudaStreamSynchronize(as_stream(stream));  // img is pageable
    delete[] img;
    if (e != cudaSuccess || e2 != cudaSuccess) return NR_ERR_CUDA;
    if (n_steps) *n_steps = steps;
    return NR_OK;
}

// One step: the projection of all cases, then one update launch per potential
// (each walks its own item range; a potential no case uses has an empty range).
static nr_status enqueue_steps(const void* table, int32_t first, int32_t count, cudaStream_t s) {
    const int fp_blocks = persistent_blocks((const void*)fp_batch_kernel, 128, 0);
    const int ub0 = persistent_blocks((const void*)update_batch_kernel<NR_POT_Q2>, 256, 0);
    const int ub1 = persistent_blocks((const void*)update_batch_kernel<NR_POT_LANGE>, 256, 0);
    const int ub2 = persistent_blocks((const void*)update_batch_kernel<NR_POT_HYPERBOLA>, 256, 0);
    const int ub3 = persistent_blocks((const void*)update_batch_kernel<NR_POT_HUBER>, 256, 0);
    const dim3 ut(UTX, UTY);
    for (int32_t k = first; k < first + count; k++) {
        fp_batch_kernel<<<fp_blocks, dim3(32, 4), 0, s>>>(table, k);
        update_batch_kernel<NR_POT_Q2><<<ub0, ut, 0, s>>>(table, k);
        update_batch_kernel<NR_POT_LANGE><<<ub1, ut, 0, s>>>(table, k);
        update_batch_kernel<NR_POT_HYPERBOLA><<<ub2, ut, 0, s>>>(table, k);
        update_batch_kernel<NR_POT_HUBER><<<ub3, ut, 0, s>>>(table, k);
    }
    return launch_status();
}

NR_API nr_status nr_batch_step(const void* table, int32_t step, void* stream) {
    if (!table || step < 0) return NR_ERR_BAD_ARGUMENT;
    return enqueue_steps(table, step, 1, as_stream(stream));
}

NR_API nr_status nr_batch_finish(const void* table, void* stream) {
    if (!table) return NR_ERR_BAD_ARGUMENT;
    finish_kernel<<<1024, 256, 0, as_stream(stream)>>>(table);
    return launch_status();
}

NR_API nr_status nr_batch_graph_create(const void* table, int32_t n_steps, void* stream,
                                       void** graph) {
    if (!table || n_steps < 1 || !graph || !stream) return NR_ERR_BAD_ARGUMENT;
    *graph = nullptr;
    cudaStream_t s = as_stream(stream);
    // occupancy queries happen before the capture starts
    persistent_blocks((const void*)fp_batch_kernel, 128, 0);
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return NR_ERR_CUDA;
    nr_status st = enqueue_steps(table, 0, n_steps, s);
    if (st == NR_OK) {
        finish_kernel<<<1024, 256, 0, s>>>(table);
        st = launch_status();
    }
    return finish_capture(s, st, graph);
}
