// objective.cu -- FP64 penalized-likelihood objective of the device-resident
// path (the reference has no objective; the nearest is the ML cost of
// ReconDBT/ML_dbt.m:88-106):
//
//   data    = sum_i (ybar_i + r_i - y_i log(ybar_i + r_i)),  ybar = b exp(-FP_cos(x))
//   penalty = 1/2 sum_j sum_{k in N26(j)} w_jk psi(x_j - x_k)
//           = sum over neighbour pairs {j,k} inside the volume of w_jk psi(t)
//
// with psi the potential whose derivative is omega(t) t (Q2 t^2/2; Lange
// d^2(|t|/d - log(1+|t|/d)); hyperbola d^2(sqrt(1+(t/d)^2) - 1); Huber t^2/2 or
// d|t| - d^2/2).  Out-of-volume neighbours have t = 0 and psi(0) = 0.
// Per-bin and per-pair terms are summed in double: per thread, then warp
// shuffles, then a per-block partial; a single block adds the partials in a
// fixed order, so the value is deterministic.
#include <cmath>
#include <mutex>
#include <utility>

#include "reduce.cuh"
#include "siddon.cuh"

namespace nr {

__global__ void __launch_bounds__(128) data_term_kernel(
    const __grid_constant__ Geo G, const float* __restrict__ x, const float* __restrict__ angles,
    const int32_t* __restrict__ index, const float* __restrict__ y, const float* __restrict__ b,
    const float* __restrict__ r, double* __restrict__ red) {
    __shared__ ViewSrc src;
    const nr_geom& g = G.g;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int a = blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    double term = 0.0;
    if (i < g.nbx && j < g.nby) {
        float v;
        float l = 0.f;
        if (trace<0>(G, x, src.x0, src.y0, src.z0, bin_x(g, i), bin_y(g, j), -g.detectorR, &v))
            l = v * src.ct;
        const int64_t o = (int64_t)a * g.nbx * g.nby + (int64_t)j * g.nbx + i;
        const double yb = (double)b[o] * exp(-(double)l);
        const double m = yb + (r ? (double)r[o] : 0.0);
        const double yy = (double)y[o];
        term = m - (yy > 0.0 ? yy * log(m) : 0.0);
    }
    const int64_t blk = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    block_partial(term, red, blk);
}

// psi(t) in double (Lange, hyperbola): t is the exact difference of two
// floats (a double holds it), and the weights are the double values
// 1/sqrt(...), so the only roundings left are the double operations' own.
template <int POT>
__device__ __forceinline__ double psi(double t, double delta) {
    if (POT == NR_POT_Q2) return 0.5 * t * t;
    if (POT == NR_POT_LANGE) {
        const double a = fabs(t) / delta;
        return delta * delta * (a - log1p(a));
    }
    if (POT == NR_POT_HYPERBOLA) {
        // d^2 (sqrt(1+u^2) - 1) = d^2 u^2 / (sqrt(1+u^2) + 1): no cancellation
        const double u = t / delta;
        const double u2 = u * u;
        return delta * delta * (u2 / (sqrt(1.0 + u2) + 1.0));
    }
    const double a = fabs(t);
    return a <= delta ? 0.5 * t * t : delta * a - 0.5 * delta * delta;
}

struct PairW {
    double w[13];  // forward neighbours: dz=+1 (9), dz=0 dy=+1 (3), dz=0 dy=0 dx=+1 (1)
    float wh[13], wl[13];  // the same as float pairs: w = wh + wl to double precision
};

// Float-float arithmetic for the quadratic potentials: a value is hi + lo
// with |lo| far below ulp(hi).  GB300 issues FP64 at 1/64 of its FP32 rate;
// these error-free transforms keep the penalty of Q2 and Huber exact to
// about 2^-44 per term in FP32 instructions, with one conversion to double
// per voxel.  The _rn intrinsics are never contracted into FMAs, which
// would break the transforms.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp))};
}
__device__ __forceinline__ FF two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
// psi(t) for t = th + tl (the exact difference of two floats): Q2 t^2/2;
// Huber t^2/2 for |t| <= delta, else delta |t| - delta^2/2.
template <int POT>
__device__ __forceinline__ FF psi_ff(float th, float tl, float delta) {
    const float at = fabsf(th);
    const bool quad = POT == NR_POT_Q2 || at < delta ||
                      (at == delta && __fmul_rn(th, tl) <= 0.f);
    if (quad) {  // (th^2 + 2 th tl) / 2
        const FF p = two_prod(th, th);
        return {__fmul_rn(0.5f, p.hi),
                __fmul_rn(0.5f, __fadd_rn(p.lo, __fmul_rn(__fmul_rn(2.f, th), tl)))};
    }
    const float atl = th < 0.f ? -tl : tl;              // |t| = at + atl
    const FF a = two_prod(delta, at);                  // delta |th|
    const FF d2 = two_prod(delta, delta);
    const FF s = two_sum(a.hi, __fmul_rn(-0.5f, d2.hi));
    return {s.hi, __fadd_rn(s.lo, __fadd_rn(__fadd_rn(a.lo, __fmul_rn(delta, atl)),
                                             __fmul_rn(-0.5f, d2.lo)))};
}

// zxy = Vz / Vx, formed in double from the float sizes.
__host__ inline PairW make_pair_weights(double zxy) {
    PairW p;
    int k = 0;
    auto put = [&](int dx, int dy, int dz) {
        p.w[k++] = 1.0 / std::sqrt((double)(dx * dx + dy * dy) + (double)(dz * dz) * zxy * zxy);
    };
    for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) put(dx, dy, 1);
    for (int dx = -1; dx <= 1; dx++) put(dx, 1, 0);
    put(1, 0, 0);
    for (int q = 0; q < 13; q++) {
        p.wh[q] = (float)p.w[q];
        p.wl[q] = (float)(p.w[q] - (double)p.wh[q]);
    }
    return p;
}

template <int POT>
__global__ void __launch_bounds__(128) penalty_kernel(const __grid_constant__ Geo G,
                                                      const __grid_constant__ PairW W,
                                                      const float* __restrict__ x, float delta,
                                                      double* __restrict__ red) {
    const nr_geom& g = G.g;
    const int ix = blockIdx.x * 32 + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    double acc = 0.0;
    if (ix < g.nx && iy < g.ny) {
        const int64_t plane = (int64_t)g.nx * g.ny;
        const int64_t v = iz * plane + (int64_t)iy * g.nx + ix;
        const float xc = x[v];
        int k = 0;
        FF sum = {0.f, 0.f};  // Q2 / Huber: float-float sum of the voxel's terms
        auto pair = [&](int dx, int dy, int dz) {
            const int kx = ix + dx, ky = iy + dy, kz = iz + dz;
            if ((unsigned)kx < (unsigned)g.nx && (unsigned)ky < (unsigned)g.ny &&
                (unsigned)kz < (unsigned)g.nz) {
                const float xn = __ldg(x + kz * plane + (int64_t)ky * g.nx + kx);
                if (POT == NR_POT_Q2 || POT == NR_POT_HUBER) {
                    const FF t = two_sum(xc, -xn);
                    const FF ps = psi_ff<POT>(t.hi, t.lo, delta);
                    // w psi: (wh + wl)(ps.hi + ps.lo), then into the sum
                    const FF pr = two_prod(W.wh[k], ps.hi);
                    const float lo = __fadd_rn(pr.lo, __fadd_rn(__fmul_rn(W.wh[k], ps.lo),
                                                                 __fmul_rn(W.wl[k], ps.hi)));
                    const FF s2 = two_sum(sum.hi, pr.hi);
                    sum = {s2.hi, __fadd_rn(sum.lo, __fadd_rn(s2.lo, lo))};
                } else {
                    const double t = (double)xc - (double)xn;
                    acc += W.w[k] * psi<POT>(t, (double)delta);
                }
            }
            k++;
        };
#pragma unroll
        for (int dy = -1; dy <= 1; dy++)
#pragma unroll
            for (int dx = -1; dx <= 1; dx++) pair(dx, dy, 1);
#pragma unroll
        for (int dx = -1; dx <= 1; dx++) pair(dx, 1, 0);
        pair(1, 0, 0);
        if (POT == NR_POT_Q2 || POT == NR_POT_HUBER) acc = (double)sum.hi + (double)sum.lo;
    }
    const int64_t blk = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    block_partial(acc, red, blk);
}

// Fixed-order sum of n partials by one block of 1024 threads.
__global__ void __launch_bounds__(1024) final_sum_kernel(const double* __restrict__ red, int64_t n0,
                                                         int64_t n1, double* __restrict__ out) {
    __shared__ double ws[32];
    for (int part = 0; part < 2; part++) {
        const double* p = red + (part == 0 ? 0 : n0);
        const int64_t n = part == 0 ? n0 : n1;
        double s = 0.0;
        for (int64_t k = threadIdx.x; k < n; k += blockDim.x) s += p[k];
        s = warp_sum(s);
        if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = ws[threadIdx.x];
            t = warp_sum(t);
            if (threadIdx.x == 0) out[part] = t;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(1024) penalty_sum_kernel(const double* __restrict__ red,
                                                           int64_t n, double* __restrict__ out) {
    sum_partials(red, n, out);
}

static int64_t data_blocks(const nr_geom& g) {
    return (int64_t)cdiv(g.nbx, 32) * cdiv(g.nby, 4) * g.n_angles;
}
static int64_t pen_blocks(const nr_geom& g) {
    return (int64_t)cdiv(g.nx, 32) * cdiv(g.ny, 4) * g.nz;
}

int64_t objective_partials(const nr_geom& g) { return data_blocks(g) + pen_blocks(g); }

template <int POT>
static void launch_penalty_t(const nr_geom& g, float delta, const float* x, double* red,
                             cudaStream_t st) {
    dim3 blk(32, 4), grd(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz);
    penalty_kernel<POT><<<grd, blk, 0, st>>>(make_geo(g),
                                             make_pair_weights((double)g.vz / (double)g.vx), x,
                                             delta, red);
}

// The penalty alone into out[0] (out[1] of launch_objective), over red_n partials.
nr_status launch_penalty(const nr_geom& g, int pot, float delta, const float* x, double* red,
                         int64_t red_n, double* out, cudaStream_t st) {
    const int64_t np = pen_blocks(g);
    if (np > red_n) return NR_ERR_WORKSPACE;
    const float dl = pot == NR_POT_Q2 ? 1.f : delta;
    switch (pot) {
    case NR_POT_Q2: launch_penalty_t<NR_POT_Q2>(g, dl, x, red, st); break;
    case NR_POT_LANGE: launch_penalty_t<NR_POT_LANGE>(g, dl, x, red, st); break;
    case NR_POT_HYPERBOLA: launch_penalty_t<NR_POT_HYPERBOLA>(g, dl, x, red, st); break;
    case NR_POT_HUBER: launch_penalty_t<NR_POT_HUBER>(g, dl, x, red, st); break;
    default: return NR_ERR_BAD_ARGUMENT;
    }
    penalty_sum_kernel<<<1, 1024, 0, st>>>(red, np, out);
    return launch_status();
}

nr_status launch_objective(const nr_geom& g, int pot, float delta, const float* x,
                           const float* angles, const int32_t* index, const float* y,
                           const float* b, const float* r, double* red, int64_t red_n,
                           double* out, cudaStream_t st) {
    const int64_t nd = data_blocks(g), np = pen_blocks(g);
    if (nd + np > red_n) return NR_ERR_WORKSPACE;
    const Geo G = make_geo(g);
    {
        dim3 blk(32, 4), grd(cdiv(g.nbx, 32), cdiv(g.nby, 4), g.n_angles);
        data_term_kernel<<<grd, blk, 0, st>>>(G, x, angles, index, y, b, r, red);
    }
    {
        dim3 blk(32, 4), grd(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz);
        const PairW W = make_pair_weights((double)g.vz / (double)g.vx);
        const float dl = pot == NR_POT_Q2 ? 1.f : delta;
        switch (pot) {
        case NR_POT_Q2: penalty_kernel<NR_POT_Q2><<<grd, blk, 0, st>>>(G, W, x, dl, red + nd); break;
        case NR_POT_LANGE:
            penalty_kernel<NR_POT_LANGE><<<grd, blk, 0, st>>>(G, W, x, dl, red + nd);
            break;
        case NR_POT_HYPERBOLA:
            penalty_kernel<NR_POT_HYPERBOLA><<<grd, blk, 0, st>>>(G, W, x, dl, red + nd);
            break;
        case NR_POT_HUBER:
            penalty_kernel<NR_POT_HUBER><<<grd, blk, 0, st>>>(G, W, x, dl, red + nd);
            break;
        default: return NR_ERR_BAD_ARGUMENT;
        }
    }
    final_sum_kernel<<<1, 1024, 0, st>>>(red, nd, np, out);
    return launch_status();
}

}  // namespace nr

// ---------------------------------------------------------------------------
// Penalty without a workspace, for callers that may not allocate device memory.
//
// Scratch: the per-block partial sums of penalty_kernel live in this
// file-scope device array (2 MiB, one copy on every GPU that loads the
// library, kept until the process exits).  In host code the name
// g_static_partials is only a host-side stand-in; the device address is
// obtained once per device with cudaGetSymbolAddress and cached.
#define NR_STATIC_PARTIALS (1 << 18)

static __device__ __align__(256) double g_static_partials[NR_STATIC_PARTIALS];

namespace nr {

// Sum of n partials into out[0], fixed order (one block of 1024 threads).
__global__ void __launch_bounds__(1024) static_sum_kernel(const double* __restrict__ red, int64_t n,
                                                          double* __restrict__ out) {
    __shared__ double ws[32];
    double s = 0.0;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) s += red[k];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = ws[threadIdx.x];
        t = warp_sum(t);
        if (threadIdx.x == 0) out[0] = t;
    }
}

// The unique id of the current context (cuCtxGetCurrent + cuCtxGetId from
// the driver, looked up once); 0 when it cannot be had.  Ids are never
// reused within a process, so a context created after cudaDeviceReset has a
// new one.
static unsigned long long current_context_id() {
    typedef int (*get_current_fn)(void**);
    typedef int (*get_id_fn)(void*, unsigned long long*);
    static const auto fns = [] {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault,
                                             &qa) != cudaSuccess ||
            qa != cudaDriverEntryPointSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) !=
                cudaSuccess ||
            qb != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            a = b = nullptr;
        }
        return std::make_pair((get_current_fn)a, (get_id_fn)b);
    }();
    if (!fns.first || !fns.second) return 0;
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (fns.first(&ctx) != 0 || !ctx || fns.second(ctx, &id) != 0) return 0;
    return id;
}

// Device address of g_static_partials on the current device.  The first call
// on a device looks it up (cudaGetSymbolAddress) with that device current and
// caches it with the context's id; a call from another context of that
// device (after cudaDeviceReset) looks it up again.  A failed lookup leaves
// no error behind in CUDA's last-error slot, so it is not charged to a later
// call.
static double* static_partials(nr_status* st) {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static double* ptrs[kMaxDevices] = {};
    static unsigned long long ctx_ids[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        *st = NR_ERR_CUDA;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!ptrs[dev] || current_context_id() != ctx_ids[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_partials) != cudaSuccess || !p) {
            cudaGetLastError();
            ptrs[dev] = nullptr;
            *st = NR_ERR_CUDA;
            return nullptr;
        }
        ptrs[dev] = (double*)p;
        // read after the lookup: it is the lookup that makes the context current
        ctx_ids[dev] = current_context_id();
    }
    return ptrs[dev];
}

}  // namespace nr

using namespace nr;

NR_API nr_status nr_penalty_fp64_static(const nr_geom* g, const float* x, int32_t potential,
                                        float delta, double* out, void* stream) {
    if (!geom_ok(g)) return NR_ERR_BAD_GEOMETRY;
    if (!x || !out) return NR_ERR_BAD_ARGUMENT;
    if (potential < NR_POT_Q2 || potential > NR_POT_HUBER) return NR_ERR_BAD_ARGUMENT;
    if (potential != NR_POT_Q2 && !(delta > 0.f)) return NR_ERR_BAD_ARGUMENT;
    if (g->vx != g->vy || g->nz > 65535) return NR_ERR_BAD_GEOMETRY;
    const int64_t np = pen_blocks(*g);
    if (np > NR_STATIC_PARTIALS) return NR_ERR_WORKSPACE;  // volume too large for the scratch
    nr_status st = NR_OK;
    double* red = static_partials(&st);
    if (!red) return st;
    cudaStream_t s = as_stream(stream);
    const Geo G = make_geo(*g);
    const PairW W = make_pair_weights((double)g->vz / (double)g->vx);
    const float dl = potential == NR_POT_Q2 ? 1.f : delta;
    dim3 blk(32, 4), grd(cdiv(g->nx, 32), cdiv(g->ny, 4), g->nz);
    // every block overwrites its own partial: nothing to clear between calls
    switch (potential) {
    case NR_POT_Q2: penalty_kernel<NR_POT_Q2><<<grd, blk, 0, s>>>(G, W, x, dl, red); break;
    case NR_POT_LANGE: penalty_kernel<NR_POT_LANGE><<<grd, blk, 0, s>>>(G, W, x, dl, red); break;
    case NR_POT_HYPERBOLA:
        penalty_kernel<NR_POT_HYPERBOLA><<<grd, blk, 0, s>>>(G, W, x, dl, red);
        break;
    default: penalty_kernel<NR_POT_HUBER><<<grd, blk, 0, s>>>(G, W, x, dl, red); break;
    }
    static_sum_kernel<<<1, 1024, 0, s>>>(red, np, out);
    return launch_status();
}
