// cnn.cu -- the learned warm start: a 3D residual CNN (6 conv 3x3x3 layers,
// 32 channels, ReLU) in BF16 on the tensor cores (tcgen05, FP32 accumulate in
// TMEM), with its backward pass and Adam.
//
// Network, in scaled units u = s * x (s = in_scale):
//     a1 = relu(conv1(u)), a_l = relu(conv_l(a_{l-1})) l = 2..5, f = conv6(a5)
//     prediction  x_warm = x + f / s          (residual on the input volume)
// Activations are channels-last BF16 [voxel][32]; a batch of nb patches is
// stacked along z with zero padding at every patch boundary.
//
// Convolution = implicit GEMM.  An output tile is one run of 128 consecutive x
// of a (patch, z, y) row (M = 128), N = output channels, K = 27 taps x input
// channels.  For 32-channel inputs the tile reads, per (dz, dy), one strip of
// 130 input rows (x0-1 .. x0+128, zero outside the volume) into shared memory
// in the K-major core-matrix layout with rows 16 bytes apart; the three dx
// taps are the same strip read from row offsets 0, 1, 2 (descriptor start +
// 16 B), so each input row is staged 9 times per tile instead of 27.  The
// strips arrive by TMA (activations are stored in 8-channel planes so that a
// strip's K chunk is one contiguous block); a producer warp, an MMA warp and
// four epilogue warps overlap staging, MMAs and stores (conv32_tma_kernel).
// Weights of all 27 taps stay in shared memory.  1-channel inputs gather the
// 27 neighbours into one K = 32 row instead.  Weight gradients of the 32 -> 32
// layers are a GEMM over voxels on the tensor cores (wgrad32_tc_kernel); those
// of the 1-channel layers are per-tap outer products on the CUDA cores.  Both
// end in the same fixed-order reduction of per-block partials.
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "tc.cuh"
#include "tma.cuh"

namespace nr {
namespace cnn {

constexpr int C = 32;                 // hidden channels
constexpr int TM = 128;               // output voxels per tile
constexpr int SROWS = TM + 2;         // strip rows incl. the x halo
constexpr int KCH = 4;                // 16-byte K chunks per 32-channel row
constexpr int WAIT_LIMIT = 1 << 24;   // polls before a wait gives up

enum { EPI_RELU = 0, EPI_MASK = 1, EPI_RESID = 2 };

struct Dims {
    int nx, ny, nz, nb;
};

__host__ __device__ inline int64_t nvox(const Dims& d) { return (int64_t)d.nx * d.ny * d.nz * d.nb; }
__host__ __device__ inline int xtiles(const Dims& d) { return (d.nx + TM - 1) / TM; }
__host__ __device__ inline int64_t ntiles(const Dims& d) {
    return (int64_t)d.ny * d.nz * d.nb * xtiles(d);
}

// Packed BF16 B operand of one tap: N rows (output channels) x 32 K in core
// matrices [N/8][4][8 rows][16 B]: SBO = 512 B between row groups, LBO = 128 B.
__host__ __device__ inline int bpk_index(int n, int k) {
    return (n >> 3) * 256 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7);
}

// Activations (and their gradients) are BF16 in planes of 8 channels: per
// row of nx voxels (one (patch, z, y) row), four planes [c / 8][x][c % 8], so
// that one K chunk (8 channels, 16 bytes) of a run of consecutive x is one
// contiguous block -- the unit the convolution's TMA boxes move.
__host__ __device__ inline int64_t act_off(int64_t v, int c, int nx) {
    const int64_t row = v / nx;
    const int x = (int)(v - row * nx);
    return (row * KCH + (c >> 3)) * (int64_t)nx * 8 + (int64_t)x * 8 + (c & 7);
}

// Epilogue of one output row: 32 accumulator columns -> output voxel v (x of
// a row of nx voxels).
template <int EPI>
__device__ __forceinline__ void epilogue(const uint32_t* acc, int64_t v, int nx,
                                         const float* __restrict__ bias, void* out,
                                         const __nv_bfloat16* __restrict__ mask) {
    if (EPI == EPI_RESID) {
        ((float*)out)[v] = __uint_as_float(acc[0]) + bias[0];
        return;
    }
    const int64_t o0 = act_off(v, 0, nx);  // chunk q at o0 + q * nx * 8
    __align__(16) __nv_bfloat16 o[C];
    if (EPI == EPI_RELU) {
#pragma unroll
        for (int c = 0; c < C; c++)
            o[c] = __float2bfloat16(fmaxf(__uint_as_float(acc[c]) + bias[c], 0.f));
    } else {
        __align__(16) __nv_bfloat16 m[C];
#pragma unroll
        for (int q = 0; q < KCH; q++)
            ((uint4*)m)[q] = __ldg((const uint4*)(mask + o0 + (int64_t)q * nx * 8));
#pragma unroll
        for (int c = 0; c < C; c++)
            o[c] = __bfloat162float(m[c]) > 0.f ? __float2bfloat16(__uint_as_float(acc[c]))
                                                : __float2bfloat16(0.f);
    }
#pragma unroll
    for (int q = 0; q < KCH; q++)
        *(uint4*)((__nv_bfloat16*)out + o0 + (int64_t)q * nx * 8) = ((const uint4*)o)[q];
}

// Row (patch b, z, y) of tile t and its first x.
__device__ __forceinline__ void tile_pos(const Dims& d, int64_t t, int& b, int& z, int& y, int& x0) {
    const int xt = xtiles(d);
    int64_t row = t / xt;
    x0 = (int)(t - row * xt) * TM;
    y = (int)(row % d.ny);
    row /= d.ny;
    z = (int)(row % d.nz);
    b = (int)(row / d.nz);
}

// ---- conv32 on a TMA + tcgen05 pipeline -------------------------------------
// 32-channel input, NOUT = 32 (hidden / dgrad) or 16 (the last layer, output
// channel 0 real) outputs; weights: 27 packed taps of NOUT x 32.  The work is
// split between warps so that staging, MMAs and the epilogue overlap:
//   warp 4 (one lane)  producer: loads each strip by TMA -- four boxes of
//                      8 channels x 130 rows, one per 16-byte K chunk, each a
//                      contiguous block of the plane layout -- so the strip
//                      lands in the K-major core-matrix layout with zeros
//                      outside the volume in x, into a ring of TSTAGE stages
//                      ("full": the bytes landed); strips outside the volume
//                      in z or y are not loaded;
//   warp 5 (one lane)  MMA issuer: 6 MMAs per loaded strip into one of two
//                      TMEM accumulators (tiles alternate); tcgen05.commit
//                      frees the stage ("empty") and, after the tile's last
//                      strip, marks the accumulator full;
//   warps 0-3          epilogue: read their 32 TMEM lanes of the finished
//                      accumulator, hand it back ("acc empty"), then apply
//                      bias / ReLU / mask and store -- while the MMAs of the
//                      next tile run into the other accumulator.
// Every wait is bounded and also gives up once another role has aborted; a
// role that gives up flags NR_FLAG_TIMEOUT and aborts the block.  Before TMEM
// is released the issuer's MMAs are drained, and the producer waits for
// every copy it issued, so nothing is in flight when the block exits.
constexpr int PLANE = 2176;                           // one K-chunk plane: 130 rows x 16 B, 128-B aligned
constexpr int TSTRIP = KCH * PLANE;                   // 8704 bytes per staged strip
// Strips in flight per CTA.  Two CTAs per SM with 6 stages each measured
// faster than one CTA per SM with 18 (25.9 against 40.7 ms for the network on
// the clinical volume, activations then channels-last): two CTAs run two
// chains of waits.
constexpr int TSTAGE = 6;
constexpr int T_THREADS = 192;
constexpr uint32_t STRIP_TX = (uint32_t)KCH * SROWS * 16;  // bytes the four boxes deliver

struct TmaCtl {
    uint64_t full[TSTAGE], empty[TSTAGE], accf[2], acce[2], drain;
    uint32_t tslot;
    int abort;
};

// A bounded wait that also gives up once the block has aborted.
__device__ __forceinline__ bool wait_live(uint64_t* bar, uint32_t parity, volatile int* abort) {
    for (int round = 0; round < WAIT_LIMIT / 1024; round++) {
        if (tc::mbar_wait(bar, parity, 1024)) return true;
        if (*abort) return false;
    }
    return false;
}

template <int NOUT, int EPI>
__global__ void __launch_bounds__(T_THREADS) conv32_tma_kernel(
    Dims d, const __grid_constant__ CUtensorMap amap, const __nv_bfloat16* __restrict__ wpk,
    const float* __restrict__ bias, void* out, const __nv_bfloat16* __restrict__ mask,
    int* status) {
    constexpr int WBYTES = 27 * NOUT * C * 2;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;
    uint8_t* sW = smem + TSTAGE * TSTRIP;
    TmaCtl* K = (TmaCtl*)(sW + WBYTES);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int k = tid; k < WBYTES / 16; k += T_THREADS)
        ((uint4*)sW)[k] = __ldg((const uint4*)wpk + k);
    if (tid == 0) {
        for (int s = 0; s < TSTAGE; s++) {
            tc::mbar_init(&K->full[s], 1);
            tc::mbar_init(&K->empty[s], 1);
        }
        for (int a = 0; a < 2; a++) {
            tc::mbar_init(&K->accf[a], 1);
            tc::mbar_init(&K->acce[a], 4);
        }
        tc::mbar_init(&K->drain, 1);
        K->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::tmem_alloc(&K->tslot, 64);
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = K->tslot;
    const int64_t nt = ntiles(d);
    volatile int* abort = &K->abort;
    auto fail = [&]() {
        if (!*abort) atomicOr(status, NR_FLAG_TIMEOUT);
        *abort = 1;
        __threadfence_block();
    };
    if (warp == 4) {
        if (lane == 0) {
            // producer
            int64_t qg = 0, issued = 0;
            for (int64_t t = blockIdx.x; t < nt && !*abort; t += gridDim.x) {
                int b, z, y, x0;
                tile_pos(d, t, b, z, y, x0);
                for (int q = 0; q < 9; q++, qg++) {
                    const int s = (int)(qg % TSTAGE);
                    if (qg >= TSTAGE &&
                        !wait_live(&K->empty[s], (uint32_t)((qg / TSTAGE - 1) & 1), abort)) {
                        fail();
                        break;
                    }
                    const int zz = z + q / 3 - 1, yy = y + q % 3 - 1;
                    if (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny) {
                        const int row = (b * d.nz + zz) * d.ny + yy;
                        uint8_t* st = sA + s * TSTRIP;
                        tc::fence_async_smem();
                        mbar_arrive_tx(&K->full[s], STRIP_TX);
                        for (int kc = 0; kc < KCH; kc++)
                            tma_load_4d(st + kc * PLANE, &amap, 0, x0 - 1, kc, row, &K->full[s]);
                    } else {
                        mbar_arrive(&K->full[s]);
                    }
                    issued = qg + 1;
                }
            }
            // no copy may be in flight when the block exits
            for (int64_t k = issued > TSTAGE ? issued - TSTAGE : 0; k < issued; k++) {
                uint64_t* bar = &K->full[k % TSTAGE];
                if (!tc::mbar_wait(bar, (uint32_t)((k / TSTAGE) & 1), WAIT_LIMIT))
                    tc::mbar_wait(bar, (uint32_t)((k / TSTAGE) & 1), WAIT_LIMIT);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            // MMA issuer
            constexpr uint32_t idesc = tc::idesc_bf16(TM, NOUT);
            const uint32_t sw = tc::smem_u32(sW);
            int64_t qg = 0;
            int lt = 0;
            for (int64_t t = blockIdx.x; t < nt && !*abort; t += gridDim.x, lt++) {
                int b, z, y, x0;
                tile_pos(d, t, b, z, y, x0);
                const int a = lt & 1;
                if (lt >= 2 && !wait_live(&K->acce[a], (uint32_t)(((lt >> 1) - 1) & 1), abort)) {
                    fail();
                    break;
                }
                tc::fence_after();
                const uint32_t dacc = tmem + (uint32_t)(a * 32);
                bool first = true, ok = true;
                for (int q = 0; q < 9; q++, qg++) {
                    const int s = (int)(qg % TSTAGE);
                    if (!wait_live(&K->full[s], (uint32_t)((qg / TSTAGE) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    const int zz = z + q / 3 - 1, yy = y + q % 3 - 1;
                    if (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny) {
                        tc::fence_after();
                        const uint32_t sa = tc::smem_u32(sA + s * TSTRIP);
#pragma unroll
                        for (int dx = 0; dx < 3; dx++) {
                            const int tap = q * 3 + dx;
#pragma unroll
                            for (int j = 0; j < 2; j++) {
                                const uint64_t ad =
                                    tc::sdesc(sa + dx * 16 + j * 2 * PLANE, PLANE, 128);
                                const uint64_t bd =
                                    tc::sdesc(sw + tap * NOUT * C * 2 + j * 256, 128, 512);
                                tc::mma_bf16(dacc, ad, bd, idesc, first ? 0u : 1u);
                                first = false;
                            }
                        }
                        tc::commit(&K->empty[s]);
                    } else {
                        mbar_arrive(&K->empty[s]);
                    }
                }
                if (!ok) {
                    fail();
                    break;
                }
                tc::commit(&K->accf[a]);
            }
        }
    } else {
        // epilogue warps 0-3: row tid of each tile.  Test hook: the
        // workspace's second status word k + 1 > 0 makes the wait for this
        // CTA's tile k report giving up once it has in fact succeeded (its
        // MMAs are complete), so the failure path runs with nothing in flight.
        const int force_at = status[1] - 1;
        int lt = 0;
        for (int64_t t = blockIdx.x; t < nt; t += gridDim.x, lt++) {
            int b, z, y, x0;
            tile_pos(d, t, b, z, y, x0);
            const int a = lt & 1;
            bool got = wait_live(&K->accf[a], (uint32_t)((lt >> 1) & 1), abort);
            if (lt == force_at) got = false;
            if (!got) {
                if (lane == 0) fail();
                break;
            }
            tc::fence_after();
            uint32_t acc[32];
            tc::ld32(tmem, (uint32_t)(warp * 32), (uint32_t)(a * 32), acc);
            tc::fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&K->acce[a]);
            const int x = x0 + tid;
            if (x < d.nx) {
                const int64_t v = (((int64_t)b * d.nz + z) * d.ny + y) * d.nx + x;
                epilogue<EPI>(acc, v, d.nx, bias, out, mask);
            }
        }
    }
    // drain: every MMA issued has completed before TMEM is released
    __syncthreads();
    if (warp == 5 && lane == 0) tc::commit(&K->drain);
    if (!tc::mbar_wait(&K->drain, 0, WAIT_LIMIT)) tc::mbar_wait(&K->drain, 0, WAIT_LIMIT);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// 1-channel input conv (the first layer, and the back projection of the last
// layer's gradient): each output row gathers its 27 neighbours (zero outside
// its patch) x scale into one K = 32 row.  Weights: one packed 32 x 32 tile.
template <int EPI>
__global__ void __launch_bounds__(128) conv1_kernel(Dims d, const float* __restrict__ in, float scale,
                                                    const __nv_bfloat16* __restrict__ wpk,
                                                    const float* __restrict__ bias, void* out,
                                                    const __nv_bfloat16* __restrict__ mask,
                                                    int* status) {
    __shared__ __align__(1024) uint8_t sW[C * C * 2];
    __shared__ __align__(1024) uint8_t sA[KCH * TM * 16];
    __shared__ __align__(8) uint64_t bars[1];
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int k = tid; k < C * C * 2 / 16; k += 128) ((uint4*)sW)[k] = __ldg((const uint4*)wpk + k);
    if (tid == 0) tc::mbar_init(&bars[0], 1);
    if (warp == 0) tc::tmem_alloc(&tslot, 32);
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tslot;
    constexpr uint32_t idesc = tc::idesc_bf16(TM, C);
    const int64_t nt = ntiles(d);
    int ntile = 0;
    int ncommit = 0;
    bool ok = true;
    const int force_at = status[1] - 1;  // test hook, as in conv32_kernel
    for (int64_t t = blockIdx.x; t < nt; t += gridDim.x) {
        int b, z, y, x0;
        tile_pos(d, t, b, z, y, x0);
        const int x = x0 + tid;
        __align__(16) __nv_bfloat16 row[32];
#pragma unroll
        for (int k = 0; k < 32; k++) {
            float v = 0.f;
            if (k < 27) {
                const int dz = k / 9 - 1, dy = (k / 3) % 3 - 1, dx = k % 3 - 1;
                const int zz = z + dz, yy = y + dy, xx = x + dx;
                if (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny && xx >= 0 && xx < d.nx && x < d.nx)
                    v = __ldg(in + (((int64_t)b * d.nz + zz) * d.ny + yy) * d.nx + xx) * scale;
            }
            row[k] = __float2bfloat16(v);
        }
        // previous tile's MMAs have completed (waited below), so sA is free
#pragma unroll
        for (int kc = 0; kc < KCH; kc++) *(uint4*)(sA + kc * TM * 16 + tid * 16) = ((uint4*)row)[kc];
        tc::fence_async_smem();
        ok = __syncthreads_and(ok) != 0;  // uniform: every thread counts the commits alike
        if (tid == 0 && ok) {
            tc::fence_after();
            const uint32_t sa = tc::smem_u32(sA), sw = tc::smem_u32(sW);
#pragma unroll
            for (int j = 0; j < 2; j++)
                tc::mma_bf16(tmem, tc::sdesc(sa + j * 2 * TM * 16, TM * 16, 128),
                             tc::sdesc(sw + j * 256, 128, 512), idesc, j != 0);
            tc::commit(&bars[0]);
        }
        if (ok) {
            ok = tc::mbar_wait(&bars[0], (uint32_t)(ncommit & 1), WAIT_LIMIT) && ntile != force_at;
            ncommit++;
        }
        ntile++;
        tc::fence_after();
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicOr(status, NR_FLAG_TIMEOUT);
            break;
        }
        uint32_t acc[32];
        tc::ld32(tmem, (uint32_t)(warp * 32), 0, acc);
        if (x < d.nx) {
            const int64_t v = (((int64_t)b * d.nz + z) * d.ny + y) * d.nx + x;
            epilogue<EPI>(acc, v, d.nx, bias, out, mask);
        }
        tc::fence_before();
        __syncthreads();
    }
    if (tid == 0) tc::commit(&bars[0]);  // drain, as in conv32_kernel
    if (!tc::mbar_wait(&bars[0], (uint32_t)(ncommit & 1), WAIT_LIMIT))
        tc::mbar_wait(&bars[0], (uint32_t)(ncommit & 1), WAIT_LIMIT);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 32);
}

// ---------------------------------------------------------------------------
// Weight gradients (CUDA cores).  dW[tap][o][i] = sum_v g[v][o] in[v+off(tap)][i]
// over the stacked patches (zero outside each patch), db[o] = sum_v g[v][o].
// Grid: (chunk of WG_CHUNK voxels, tap 0..27; tap 27 = bias).  Each block
// writes one partial per output; wgrad_reduce_kernel adds the chunks in order.
constexpr int WG_CHUNK = 2048;
constexpr int WG_SUB = 64;

__device__ __forceinline__ float ld_act(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// Loads the shifted input (tap) and the output gradient of voxels s .. s+WG_SUB-1
// into shared memory as FP32 (zero outside each patch / past the end).
template <int NI, int NO, int GP, int XP>
__device__ __forceinline__ void wg_stage(const Dims& d, int tap, int64_t s, int64_t V,
                                         const void* __restrict__ g_, const void* __restrict__ in_,
                                         float in_scale, float (*gs)[GP], float (*xs)[XP]) {
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    for (int e = threadIdx.x; e < WG_SUB * NO; e += blockDim.x) {
        const int vi = e / NO, o = e % NO;
        const int64_t v = s + vi;
        float gv = 0.f;
        if (v < V)
            gv = NO == 1 ? ((const float*)g_)[v]
                         : ld_act((const __nv_bfloat16*)g_ + act_off(v, o, d.nx));
        gs[vi][o] = gv;
    }
    for (int e = threadIdx.x; e < WG_SUB * NI; e += blockDim.x) {
        const int vi = e / NI, i = e % NI;
        const int64_t v = s + vi;
        float xv = 0.f;
        if (v < V) {
            if (tap == 27) {
                xv = 1.f;  // the bias "tap"
            } else {
                int64_t r = v;
                const int x = (int)(r % d.nx);
                r /= d.nx;
                const int y = (int)(r % d.ny);
                r /= d.ny;
                const int z = (int)(r % d.nz);
                const int b = (int)(r / d.nz);
                const int xx = x + dx, yy = y + dy, zz = z + dz;
                if (xx >= 0 && xx < d.nx && yy >= 0 && yy < d.ny && zz >= 0 && zz < d.nz) {
                    const int64_t u = (((int64_t)b * d.nz + zz) * d.ny + yy) * d.nx + xx;
                    xv = NI == 1 ? ((const float*)in_)[u] * in_scale
                                 : ld_act((const __nv_bfloat16*)in_ + act_off(u, i, d.nx));
                }
            }
        }
        xs[vi][i] = xv;
    }
}

// 32 x 32 layers: thread -> output channel o = tid/8 and inputs i0..i0+3.
__global__ void __launch_bounds__(256) wgrad32_kernel(Dims d, const __nv_bfloat16* __restrict__ g,
                                                      const __nv_bfloat16* __restrict__ in,
                                                      float* __restrict__ partial) {
    __shared__ __align__(16) float gs[WG_SUB][C + 1];
    __shared__ __align__(16) float xs[WG_SUB][C + 4];
    const int tap = blockIdx.y;
    const int64_t V = nvox(d);
    const int64_t v0 = (int64_t)blockIdx.x * WG_CHUNK;
    const int o = threadIdx.x >> 3, i0 = (threadIdx.x & 7) * 4;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    for (int64_t s = v0; s < v0 + WG_CHUNK && s < V; s += WG_SUB) {
        wg_stage<C, C, C + 1, C + 4>(d, tap, s, V, g, in, 1.f, gs, xs);
        __syncthreads();
#pragma unroll 8
        for (int vi = 0; vi < WG_SUB; vi++) {
            const float gv = gs[vi][o];
            const float4 xv = *(const float4*)&xs[vi][i0];
            a0 = fmaf(gv, xv.x, a0);
            a1 = fmaf(gv, xv.y, a1);
            a2 = fmaf(gv, xv.z, a2);
            a3 = fmaf(gv, xv.w, a3);
        }
        __syncthreads();
    }
    const int64_t nchunk = gridDim.x;
    const int64_t base = ((int64_t)tap * C * C + o * C + i0) * nchunk + blockIdx.x;
    partial[base] = a0;
    partial[base + nchunk] = a1;
    partial[base + 2 * nchunk] = a2;
    partial[base + 3 * nchunk] = a3;
}

// Thin layers (NI = 1 or NO = 1): 32 outputs per tap, one per thread of 32.
template <int NI, int NO>
__global__ void __launch_bounds__(32) wgrad_thin_kernel(Dims d, const void* __restrict__ g_,
                                                        const void* __restrict__ in_,
                                                        float in_scale,
                                                        float* __restrict__ partial) {
    __shared__ float gs[WG_SUB][NO + 1];
    __shared__ float xs[WG_SUB][NI + 1];
    const int tap = blockIdx.y;
    const int64_t V = nvox(d);
    const int64_t v0 = (int64_t)blockIdx.x * WG_CHUNK;
    const int oi = threadIdx.x;  // NI * NO == 32
    const int o = oi / NI, i = oi % NI;
    float acc = 0.f;
    for (int64_t s = v0; s < v0 + WG_CHUNK && s < V; s += WG_SUB) {
        wg_stage<NI, NO, NO + 1, NI + 1>(d, tap, s, V, g_, in_, in_scale, gs, xs);
        __syncthreads();
        for (int vi = 0; vi < WG_SUB; vi++) acc = fmaf(gs[vi][o], xs[vi][i], acc);
        __syncthreads();
    }
    partial[((int64_t)tap * 32 + oi) * gridDim.x + blockIdx.x] = acc;
}

// ---- Weight gradient of the 32 -> 32 layers on the tensor cores -------------
// dW[tap][o][i] = sum_v g[v][o] a[v + off(tap)][i] as a GEMM with M = (tap, i),
// N = o, K = voxels: C[(tap, i)][o] = sum_v A[(tap, i)][v] B[o][v] with
// A = the input activations shifted by the tap and B = the output gradient.
// Per block of 128 consecutive voxels of a (patch, z, y) row (the K block),
// one lane loads by TMA the nine input strips (rows z+dz, y+dy; x0-1 ..
// x0+128) and the gradient strip; the four warps transpose 8 x 8 blocks
// (ldmatrix .trans, stmatrix) from the activations' plane layout [x][8 channels]
// into the K-major operand layout [channel][8 x], the tap's x shift being the
// source row offset; and one lane issues, per M block of 4 taps (7 blocks: 27
// taps and a block of ones whose row sums give the bias gradient), 8 MMAs of
// K = 16 into that block's TMEM accumulator (32 columns).  A and B buffers are
// double-buffered against the MMAs by tcgen05.commit barriers.  Each CTA adds
// its K blocks into TMEM and writes one partial per weight, in the layout of
// wgrad32_kernel, for the same fixed-order reduction.  Out-of-volume strips
// are zeros.  Every wait is bounded; a wait that gives up flags
// NR_FLAG_TIMEOUT, stops further copies and MMAs, and the MMAs issued and the
// copies in flight are waited for before TMEM is released.
constexpr int WT_GROUP = 2048;                        // bytes per 8-row group of a K-major operand (16 K chunks)
constexpr int WT_ABUF = 16 * WT_GROUP;                // A: 4 taps x 32 channels x 128 voxels
constexpr int WT_BBUF = 4 * WT_GROUP;                 // B: 32 channels x 128 voxels
constexpr int WT_PLANE = 2176;                        // staged plane: 130 rows x 16 B, 128-B aligned
constexpr int WT_STRIP = KCH * WT_PLANE;
constexpr uint32_t WT_STRIP_TX = (uint32_t)KCH * SROWS * 16;
constexpr int WT_SMEM = 10 * WT_STRIP + 2 * WT_ABUF + 2 * WT_BBUF + 128;

__device__ __forceinline__ void ldsm_x4_trans(uint32_t addr, uint32_t* r) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}
__device__ __forceinline__ void stsm_x4(uint32_t addr, const uint32_t* r) {
    asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1, %2, %3, %4};" ::"r"(addr),
                 "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3])
                 : "memory");
}

// One warp transposes a staged strip (rows = x, 4 planes of 8 channels) into
// slot `slot` (32 rows) of a K-major operand: operand row 8p + c, K chunk b
// (x = 8b .. 8b+7) <- strip plane p, rows shift + 8b .. shift + 8b + 7.  The
// warp does units u0, u0 + step, ... of the 16 units (plane p = u / 4, chunks
// 4 (u % 4) .. + 3; one x4 instruction pair each).
__device__ __forceinline__ void wt_transpose(const uint8_t* strip, int shift, uint8_t* op,
                                             int slot, int u0, int step, int lane) {
    for (int u = u0; u < 16; u += step) {
        const int p = u >> 2, b = 4 * (u & 3) + (lane >> 3), rr = lane & 7;
        uint32_t r[4];
        ldsm_x4_trans(tc::smem_u32(strip + p * WT_PLANE + (shift + 8 * b + rr) * 16), r);
        stsm_x4(tc::smem_u32(op + (slot * 4 + p) * WT_GROUP + b * 128 + rr * 16), r);
    }
}
// The same slot filled with a constant 16-bit pattern (0: zeros, 0x3F80: ones).
__device__ __forceinline__ void wt_fill(uint8_t* op, int slot, uint32_t pat, int t0, int nt) {
    const uint4 v = make_uint4(pat * 0x10001u, pat * 0x10001u, pat * 0x10001u, pat * 0x10001u);
    uint4* q = (uint4*)(op + slot * 4 * WT_GROUP);
    for (int k = t0; k < 4 * WT_GROUP / 16; k += nt) q[k] = v;
}

__global__ void __launch_bounds__(128, 1) wgrad32_tc_kernel(Dims d,
                                                            const __grid_constant__ CUtensorMap amap,
                                                            const __grid_constant__ CUtensorMap gmap,
                                                            float* __restrict__ partial,
                                                            int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* stg = smem;                                   // 9 input strips + the gradient strip
    uint8_t* abuf = smem + 10 * WT_STRIP;                   // 2 x A
    uint8_t* bbuf = abuf + 2 * WT_ABUF;                     // 2 x B
    uint64_t* bars = (uint64_t*)(bbuf + 2 * WT_BBUF);       // sbar, abar[2], drain
    uint32_t* tslot = (uint32_t*)(bars + 4);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int k = 0; k < 4; k++) tc::mbar_init(&bars[k], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::tmem_alloc(tslot, 256);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const int64_t nt = ntiles(d);
    const int force_at = status[1] - 1;  // test hook: the wait for K block k gives up
    constexpr uint32_t idesc = tc::idesc_bf16(TM, C);
    bool ok = true;
    int kb = 0, c = 0;
    int64_t staged = -1;  // the K block whose copies were issued and not yet waited for
    for (int64_t t = blockIdx.x; t < nt; t += gridDim.x, kb++) {
        int b, z, y, x0;
        tile_pos(d, t, b, z, y, x0);
        if (tid == 0) {
            uint32_t bytes = WT_STRIP_TX;  // the gradient strip
            for (int q = 0; q < 9; q++) {
                const int zz = z + q / 3 - 1, yy = y + q % 3 - 1;
                if (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny) bytes += WT_STRIP_TX;
            }
            tc::fence_async_smem();
            mbar_arrive_tx(&bars[0], bytes);
            const int grow = (b * d.nz + z) * d.ny + y;
            for (int kc = 0; kc < KCH; kc++)
                tma_load_4d(stg + 9 * WT_STRIP + kc * WT_PLANE, &gmap, 0, x0 - 1, kc, grow, &bars[0]);
            for (int q = 0; q < 9; q++) {
                const int zz = z + q / 3 - 1, yy = y + q % 3 - 1;
                if (!(zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny)) continue;
                const int row = (b * d.nz + zz) * d.ny + yy;
                for (int kc = 0; kc < KCH; kc++)
                    tma_load_4d(stg + q * WT_STRIP + kc * WT_PLANE, &amap, 0, x0 - 1, kc, row,
                                &bars[0]);
            }
        }
        staged = kb;
        bool got = tc::mbar_wait(&bars[0], (uint32_t)(kb & 1), WAIT_LIMIT) && kb != force_at;
        if (!__syncthreads_and(got)) {
            ok = false;
            break;
        }
        staged = -1;
        for (int mb = 0; mb < 7; mb++, c++) {
            const int j = c & 1;
            // the MMAs of use c - 2 of this A buffer (and, at mb 0, every MMA
            // of K block kb - 2, the last reader of this B buffer) are done;
            // a warp in which a wait gave up writes nothing (the transposes are
            // warp-collective, so the decision is the warp's)
            if (c >= 2 &&
                !__all_sync(0xffffffffu,
                            tc::mbar_wait(&bars[1 + j], (uint32_t)(((c >> 1) - 1) & 1), WAIT_LIMIT)))
                ok = false;
            uint8_t* A = abuf + j * WT_ABUF;
            uint8_t* Bm = bbuf + (kb & 1) * WT_BBUF;
            if (ok && mb == 0) wt_transpose(stg + 9 * WT_STRIP, 1, Bm, 0, warp, 4, lane);
            for (int sl = 0; sl < 4 && ok; sl++) {
                const int tap = 4 * mb + sl;
                if (tap == 27) {
                    wt_fill(A, sl, 0x3F80u, tid, 128);  // ones: the bias gradient
                    continue;
                }
                const int q = tap / 3, dx = tap % 3;
                const int zz = z + q / 3 - 1, yy = y + q % 3 - 1;
                if (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny)
                    wt_transpose(stg + q * WT_STRIP, dx, A, sl, warp, 4, lane);
                else
                    wt_fill(A, sl, 0u, tid, 128);
            }
            tc::fence_async_smem();
            if (!__syncthreads_and(ok)) {
                ok = false;
                break;
            }
            if (tid == 0) {
                tc::fence_after();
                const uint32_t sa = tc::smem_u32(A), sb = tc::smem_u32(Bm);
#pragma unroll
                for (int st = 0; st < TM / 16; st++)
                    tc::mma_bf16(tmem + (uint32_t)(mb * 32), tc::sdesc(sa + st * 256, 128, WT_GROUP),
                                 tc::sdesc(sb + st * 256, 128, WT_GROUP), idesc,
                                 (kb > 0 || st > 0) ? 1u : 0u);
                tc::commit(&bars[1 + j]);
            }
        }
        if (!ok) break;
        tc::fence_async_smem();  // this block's reads of the staging precede the next copies
        __syncthreads();
    }
    if (!ok && tid == 0) atomicOr(status, NR_FLAG_TIMEOUT);
    // copies still in flight land, and every MMA issued completes, before TMEM goes
    if (tid == 0 && staged >= 0 && !tc::mbar_wait(&bars[0], (uint32_t)(staged & 1), WAIT_LIMIT))
        tc::mbar_wait(&bars[0], (uint32_t)(staged & 1), WAIT_LIMIT);
    if (tid == 0) tc::commit(&bars[3]);
    if (!tc::mbar_wait(&bars[3], 0, WAIT_LIMIT)) tc::mbar_wait(&bars[3], 0, WAIT_LIMIT);
    tc::fence_after();
    if (ok && kb > 0) {
        // TMEM lane 32 w + l = (tap 4 mb + w, input channel l), column o
        const int64_t nchunk = gridDim.x;
        for (int mb = 0; mb < 7; mb++) {
            uint32_t acc[32];
            tc::ld32(tmem, (uint32_t)(warp * 32), (uint32_t)(mb * 32), acc);
            const int tap = 4 * mb + warp;
            for (int o = 0; o < C; o++)
                partial[(((int64_t)tap * C + o) * C + lane) * nchunk + blockIdx.x] =
                    __uint_as_float(acc[o]);
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 256);
}

// grad[tap][o][i] (and grad_b[o] from tap 27, i = 0) = sum over chunks, in order.
__global__ void wgrad_reduce_kernel(const float* __restrict__ partial, int64_t nchunk, int nout,
                                    int ni, float* __restrict__ gw, float* __restrict__ gb) {
    const int64_t n = 28LL * nout;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        const float* p = partial + e * nchunk;
        double s = 0.0;
        for (int64_t c = 0; c < nchunk; c++) s += p[c];
        const int tap = (int)(e / nout), oi = (int)(e % nout);
        if (tap < 27) gw[e] = (float)s;
        else if (oi % ni == 0) gb[oi / ni] = (float)s;
    }
}

// ---------------------------------------------------------------------------
// Packing FP32 master weights W[tap][o][i] into the BF16 B operands.
// mode 0: forward of a 32-input layer: tap t, row n = o (NOUT rows, o >= NO zero), k = i.
// mode 1: dgrad of a 32-output layer (input gradient has NO = 32 channels):
//         tap t' , row n = i, k = o, from W[26 - t'] (flipped).
// mode 2: forward of the 1-input layer: one tile, row n = o, k = tap.
// mode 3: dgrad of the 1-output layer as a 1-channel conv: row n = i, k = tap',
//         from W[26 - tap'][0][i].
__global__ void pack_kernel(const float* __restrict__ w, int mode, int NI, int NO, int NOUT,
                            __nv_bfloat16* __restrict__ out) {
    const int per_tap = NOUT * C;
    const int total = (mode == 2 || mode == 3) ? C * C : 27 * per_tap;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        float v = 0.f;
        int dst;
        if (mode == 0) {
            const int t = e / per_tap, r = e % per_tap, n = r / C, k = r % C;
            if (n < NO && k < NI) v = w[((int64_t)t * NO + n) * NI + k];
            dst = t * per_tap + bpk_index(n, k);
        } else if (mode == 1) {
            const int t = e / per_tap, r = e % per_tap, n = r / C, k = r % C;
            if (n < NI && k < NO) v = w[((int64_t)(26 - t) * NO + k) * NI + n];
            dst = t * per_tap + bpk_index(n, k);
        } else if (mode == 2) {
            const int n = e / C, k = e % C;
            if (k < 27 && n < NO) v = w[((int64_t)k * NO + n) * NI + 0];
            dst = bpk_index(n, k);
        } else {
            const int n = e / C, k = e % C;
            if (k < 27 && n < NI) v = w[((int64_t)(26 - k) * NO + 0) * NI + n];
            dst = bpk_index(n, k);
        }
        out[dst] = __float2bfloat16(v);
    }
}

// Loss 1/V sum (f - r)^2 (per-block FP64 partials) and its gradient 2(f - r)/V.
__global__ void loss_kernel(const float* __restrict__ f, const float* __restrict__ r, int64_t V,
                            float* __restrict__ g, double* __restrict__ partial) {
    __shared__ double ws[8];
    double s = 0.0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V;
         v += (int64_t)gridDim.x * blockDim.x) {
        const float e = f[v] - r[v];
        g[v] = 2.f * e / (float)V;
        s += (double)e * e;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += ws[k];
        partial[blockIdx.x] = t;
    }
}

__global__ void loss_final_kernel(const double* __restrict__ partial, int n, int64_t V,
                                  double* __restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < n; k++) t += partial[k];
        out[0] = t / (double)V;
    }
}

// Adam (Kingma & Ba 2015) with bias correction, FP32 master parameters.
__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const float gk = g[k];
        const float mk = b1 * m[k] + (1.f - b1) * gk;
        const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
        m[k] = mk;
        v[k] = vk;
        p[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
    }
}

// x_warm = x + f / s (and a non-negativity clamp, the OSTR constraint).
__global__ void residual_out_kernel(const float* __restrict__ x, const float* __restrict__ f,
                                    float inv_s, int64_t V, float* __restrict__ out) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V;
         v += (int64_t)gridDim.x * blockDim.x)
        out[v] = fmaxf(x[v] + f[v] * inv_s, 0.f);
}

}  // namespace cnn
}  // namespace nr

// ---------------------------------------------------------------------------
// Host side: parameter layout, workspace layout, forward / backward sequencing.
namespace nr {
namespace cnn {

struct Layer {
    int ni, no;
};
constexpr Layer LAYERS[6] = {{1, C}, {C, C}, {C, C}, {C, C}, {C, C}, {C, 1}};

// FP32 parameters: for each layer W[27][no][ni] then b[no].
static void param_offsets(int64_t* w, int64_t* b, int64_t* total) {
    int64_t o = 0;
    for (int l = 0; l < 6; l++) {
        w[l] = o;
        o += 27LL * LAYERS[l].no * LAYERS[l].ni;
        b[l] = o;
        o += LAYERS[l].no;
    }
    *total = o;
}

constexpr size_t PK_HID = 27 * C * C * 2;   // packed 32 -> 32 taps
constexpr size_t PK_LAST = 27 * 16 * C * 2; // packed 32 -> 1 (16 rows)
constexpr size_t PK_ONE = C * C * 2;        // packed 1-channel tile

struct WSL {
    size_t status, pk_fwd[6], pk_bwd[6], act[5], f, r, g6, dpre[2], part, grad, lpart, lout, total;
    int64_t nchunk, lblocks;
};

static size_t al(size_t v) { return (v + 255) & ~(size_t)255; }

static WSL layout(const Dims& d, bool training) {
    WSL L{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = al(o + bytes);
        return at;
    };
    const int64_t V = nvox(d);
    int64_t wo[6], bo[6], P;
    param_offsets(wo, bo, &P);
    L.status = take(256);
    L.pk_fwd[0] = take(PK_ONE);
    for (int l = 1; l < 5; l++) L.pk_fwd[l] = take(PK_HID);
    L.pk_fwd[5] = take(PK_LAST);
    const int nact = training ? 5 : 2;
    for (int k = 0; k < nact; k++) L.act[k] = take((size_t)V * C * 2);
    L.f = take((size_t)V * 4);
    L.nchunk = (V + WG_CHUNK - 1) / WG_CHUNK;
    L.lblocks = 1024;
    if (training) {
        for (int l = 1; l < 5; l++) L.pk_bwd[l] = take(PK_HID);
        L.pk_bwd[5] = take(PK_ONE);
        L.r = take((size_t)V * 4);
        L.g6 = take((size_t)V * 4);
        L.dpre[0] = take((size_t)V * C * 2);
        L.dpre[1] = take((size_t)V * C * 2);
        L.part = take((size_t)28 * C * C * L.nchunk * 4);
        L.grad = take((size_t)P * 4);
        L.lpart = take((size_t)L.lblocks * 8);
        L.lout = take(8);
    }
    L.total = o;
    return L;
}

static int sm_count() {
    int dev = 0, n = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
}

}  // namespace cnn
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encode_fn();
namespace cnn {

// The TMA map of an activation tensor (act_off's layout) seen as (8 channels,
// nx, 4 K chunks, R rows): one box is one K chunk of 130 consecutive x, a
// contiguous 2080-byte block away from the row ends (zeros outside them).
static bool act_map(const Dims& d, const __nv_bfloat16* in, CUtensorMap* map) {
    auto enc = tensor_map_encode_fn();
    if (!enc || ((uintptr_t)in & 15) != 0) return false;
    const cuuint64_t rows = (cuuint64_t)d.ny * d.nz * d.nb;
    const cuuint64_t dims[4] = {8, (cuuint64_t)d.nx, (cuuint64_t)KCH, rows};
    const cuuint64_t strides[3] = {16, (cuuint64_t)d.nx * 16, (cuuint64_t)d.nx * C * 2};
    const cuuint32_t box[4] = {8, (cuuint32_t)SROWS, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)in, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NOUT, int EPI>
static nr_status launch_conv32(const Dims& d, const __nv_bfloat16* in, const __nv_bfloat16* wpk,
                               const float* bias, void* out, const __nv_bfloat16* mask,
                               int* status, cudaStream_t s) {
    CUtensorMap map;
    if (!act_map(d, in, &map)) return NR_ERR_CUDA;  // the input cannot be described for TMA
    const size_t smem = (size_t)TSTAGE * TSTRIP + 27 * NOUT * C * 2 + sizeof(TmaCtl);
    if (cudaFuncSetAttribute(conv32_tma_kernel<NOUT, EPI>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return NR_ERR_CUDA;
    const int64_t nt = ntiles(d);
    const int grid = (int)(nt < (int64_t)sm_count() * 2 ? nt : (int64_t)sm_count() * 2);
    conv32_tma_kernel<NOUT, EPI><<<grid, T_THREADS, smem, s>>>(d, map, wpk, bias, out, mask,
                                                               status);
    return launch_status();
}

template <int EPI>
static nr_status launch_conv1(const Dims& d, const float* in, float scale,
                              const __nv_bfloat16* wpk, const float* bias, void* out,
                              const __nv_bfloat16* mask, int* status, cudaStream_t s) {
    const int64_t nt = ntiles(d);
    const int grid = (int)(nt < (int64_t)sm_count() * 4 ? nt : (int64_t)sm_count() * 4);
    conv1_kernel<EPI><<<grid, 128, 0, s>>>(d, in, scale, wpk, bias, out, mask, status);
    return launch_status();
}

static void pack(const float* w, int mode, int ni, int no, int nout, __nv_bfloat16* out,
                 cudaStream_t s) {
    pack_kernel<<<64, 256, 0, s>>>(w, mode, ni, no, nout, out);
}

// Forward through layer 6: f = conv6(a5) in `f`; activations in `acts`
// (5 buffers when `keep`, else 2 ping-pong buffers).
static nr_status forward(const Dims& d, const float* params, const float* x, float s,
                         char* ws, const WSL& L, bool keep, cudaStream_t st) {
    int64_t wo[6], bo[6], P;
    param_offsets(wo, bo, &P);
    int* status = (int*)(ws + L.status);
    auto pkf = [&](int l) { return (__nv_bfloat16*)(ws + L.pk_fwd[l]); };
    pack(params + wo[0], 2, 1, C, C, pkf(0), st);
    for (int l = 1; l < 5; l++) pack(params + wo[l], 0, C, C, C, pkf(l), st);
    pack(params + wo[5], 0, C, 1, 16, pkf(5), st);
    auto act = [&](int l) {  // output of layer l (0-based, l < 5)
        return (__nv_bfloat16*)(ws + L.act[keep ? l : (l & 1)]);
    };
    nr_status e;
    if ((e = launch_conv1<EPI_RELU>(d, x, s, pkf(0), params + bo[0], act(0), nullptr, status, st)) != NR_OK)
        return e;
    for (int l = 1; l < 5; l++)
        if ((e = launch_conv32<C, EPI_RELU>(d, act(l - 1), pkf(l), params + bo[l], act(l), nullptr,
                                            status, st)) != NR_OK)
            return e;
    return launch_conv32<16, EPI_RESID>(d, act(4), pkf(5), params + bo[5], ws + L.f, nullptr,
                                        status, st);
}

__global__ void target_kernel(const float* __restrict__ x, const float* __restrict__ t, float s,
                              int64_t V, float* __restrict__ r) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V;
         v += (int64_t)gridDim.x * blockDim.x)
        r[v] = s * (t[v] - x[v]);
}

static nr_status wgrad(const Dims& d, int l, const void* g, const void* in, float s, char* ws,
                       const WSL& L, float* grad, int* status, cudaStream_t st) {
    int64_t wo[6], bo[6], P;
    param_offsets(wo, bo, &P);
    float* part = (float*)(ws + L.part);
    const dim3 grid((unsigned)L.nchunk, 28);
    int nout, ni;
    if (l == 0) {
        wgrad_thin_kernel<1, C><<<grid, 32, 0, st>>>(d, g, in, s, part);
        nout = C;
        ni = 1;
    } else if (l == 5) {
        wgrad_thin_kernel<C, 1><<<grid, 32, 0, st>>>(d, g, in, 1.f, part);
        nout = C;
        ni = C;
    } else {
        // the tensor-core form: one partial per CTA (at most L.nchunk CTAs)
        CUtensorMap am, gm;
        if (!act_map(d, (const __nv_bfloat16*)in, &am) || !act_map(d, (const __nv_bfloat16*)g, &gm))
            return NR_ERR_CUDA;
        if (cudaFuncSetAttribute(wgrad32_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 WT_SMEM) != cudaSuccess)
            return NR_ERR_CUDA;
        const int64_t nt = ntiles(d);
        int64_t nch = nt < (int64_t)sm_count() ? nt : (int64_t)sm_count();
        if (nch > L.nchunk) nch = L.nchunk;
        wgrad32_tc_kernel<<<(unsigned)nch, 128, WT_SMEM, st>>>(d, am, gm, part, status);
        wgrad_reduce_kernel<<<(28 * C * C + 255) / 256, 256, 0, st>>>(part, nch, C * C, C,
                                                                      grad + wo[l], grad + bo[l]);
        return launch_status();
    }
    wgrad_reduce_kernel<<<(28 * nout + 255) / 256, 256, 0, st>>>(part, L.nchunk, nout, ni,
                                                                 grad + wo[l], grad + bo[l]);
    return launch_status();
}

static nr_status loss_grad(const Dims& d, const float* params, const float* x, const float* target,
                           float s, float* grad, char* ws, const WSL& L, cudaStream_t st) {
    const int64_t V = nvox(d);
    int64_t wo[6], bo[6], P;
    param_offsets(wo, bo, &P);
    int* status = (int*)(ws + L.status);
    nr_status e;
    if ((e = forward(d, params, x, s, ws, L, true, st)) != NR_OK) return e;
    float* r = (float*)(ws + L.r);
    float* g6 = (float*)(ws + L.g6);
    target_kernel<<<1024, 256, 0, st>>>(x, target, s, V, r);
    loss_kernel<<<(unsigned)L.lblocks, 256, 0, st>>>((const float*)(ws + L.f), r, V, g6,
                                                      (double*)(ws + L.lpart));
    loss_final_kernel<<<1, 32, 0, st>>>((const double*)(ws + L.lpart), (int)L.lblocks, V,
                                        (double*)(ws + L.lout));
    auto act = [&](int l) { return (const __nv_bfloat16*)(ws + L.act[l]); };
    auto dpre = [&](int k) { return (__nv_bfloat16*)(ws + L.dpre[k & 1]); };
    auto pkb = [&](int l) { return (__nv_bfloat16*)(ws + L.pk_bwd[l]); };
    for (int l = 1; l < 5; l++) pack(params + wo[l], 1, C, C, C, pkb(l), st);
    pack(params + wo[5], 3, C, 1, C, pkb(5), st);
    // layer 6: weight gradient and the masked input gradient dpre5
    if ((e = wgrad(d, 5, g6, act(4), 1.f, ws, L, grad, status, st)) != NR_OK) return e;
    if ((e = launch_conv1<EPI_MASK>(d, g6, 1.f, pkb(5), nullptr, dpre(4), act(4), status, st)) !=
        NR_OK)
        return e;
    // layers 5..2: dpre_l lives in dpre(l-1)
    for (int l = 4; l >= 1; l--) {
        if ((e = wgrad(d, l, dpre(l), act(l - 1), 1.f, ws, L, grad, status, st)) != NR_OK) return e;
        if ((e = launch_conv32<C, EPI_MASK>(d, dpre(l), pkb(l), nullptr, dpre(l - 1), act(l - 1),
                                            status, st)) != NR_OK)
            return e;
    }
    return wgrad(d, 0, dpre(0), x, s, ws, L, grad, status, st);
}

}  // namespace cnn
}  // namespace nr

using namespace nr;
using namespace nr::cnn;

static bool dims_ok(const nr_cnn_dims* d) {
    return d && d->nx > 0 && d->ny > 0 && d->nz > 0 && d->nb > 0 &&
           (int64_t)d->nx * d->ny * d->nz * d->nb < ((int64_t)1 << 31);
}

static Dims to_dims(const nr_cnn_dims* d) { return Dims{d->nx, d->ny, d->nz, d->nb}; }

NR_API nr_status nr_cnn_param_count(int64_t* n) {
    if (!n) return NR_ERR_BAD_ARGUMENT;
    int64_t wo[6], bo[6];
    param_offsets(wo, bo, n);
    return NR_OK;
}

NR_API nr_status nr_cnn_workspace_size(const nr_cnn_dims* d, int32_t training, size_t* bytes) {
    if (!dims_ok(d) || !bytes) return NR_ERR_BAD_ARGUMENT;
    *bytes = layout(to_dims(d), training != 0).total;
    return NR_OK;
}

NR_API nr_status nr_cnn_forward(const nr_cnn_dims* d, const float* params, const float* x,
                                float in_scale, float* x_out, void* ws, size_t ws_bytes,
                                void* stream) {
    if (!dims_ok(d) || !params || !x || !x_out || !(in_scale > 0.f)) return NR_ERR_BAD_ARGUMENT;
    const Dims D = to_dims(d);
    const WSL L = layout(D, false);
    if (!ws || ws_bytes < L.total || ((uintptr_t)ws & 255)) return NR_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    nr_status e = forward(D, params, x, in_scale, (char*)ws, L, false, st);
    if (e != NR_OK) return e;
    residual_out_kernel<<<1024, 256, 0, st>>>(x, (const float*)((char*)ws + L.f), 1.f / in_scale,
                                              nvox(D), x_out);
    return launch_status();
}

NR_API nr_status nr_cnn_loss_grad(const nr_cnn_dims* d, const float* params, const float* x,
                                  const float* target, float in_scale, float* grad, double* loss,
                                  void* ws, size_t ws_bytes, void* stream) {
    if (!dims_ok(d) || !params || !x || !target || !(in_scale > 0.f)) return NR_ERR_BAD_ARGUMENT;
    const Dims D = to_dims(d);
    const WSL L = layout(D, true);
    if (!ws || ws_bytes < L.total || ((uintptr_t)ws & 255)) return NR_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    char* w = (char*)ws;
    float* g = grad ? grad : (float*)(w + L.grad);
    nr_status e = loss_grad(D, params, x, target, in_scale, g, w, L, st);
    if (e != NR_OK) return e;
    if (loss &&
        cudaMemcpyAsync(loss, w + L.lout, 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return NR_ERR_CUDA;
    return NR_OK;
}

NR_API nr_status nr_cnn_adam(float* params, float* m, float* v, const float* grad, int64_t n,
                             int32_t step, float lr, void* stream) {
    if (!params || !m || !v || !grad || n <= 0 || step < 1 || !(lr > 0.f)) return NR_ERR_BAD_ARGUMENT;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<256, 256, 0, as_stream(stream)>>>(params, m, v, grad, n, lr, b1, b2, 1e-8f, c1,
                                                    c2);
    return launch_status();
}

NR_API nr_status nr_cnn_train_step(const nr_cnn_dims* d, float* params, float* adam_m,
                                   float* adam_v, int32_t step, float lr, const float* x,
                                   const float* target, float in_scale, double* loss, void* ws,
                                   size_t ws_bytes, void* stream) {
    nr_status e = nr_cnn_loss_grad(d, params, x, target, in_scale, nullptr, loss, ws, ws_bytes,
                                   stream);
    if (e != NR_OK) return e;
    const WSL L = layout(to_dims(d), true);
    int64_t P;
    nr_cnn_param_count(&P);
    return nr_cnn_adam(params, adam_m, adam_v, (const float*)((char*)ws + L.grad), P, step, lr,
                       stream);
}

NR_API nr_status nr_cnn_check(void* ws, int32_t* flags, void* stream) {
    if (!ws || !flags) return NR_ERR_BAD_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    int v = 0;
    if (cudaMemcpyAsync(&v, ws, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return NR_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return NR_ERR_CUDA;
    *flags = v;
    if (v) cudaMemsetAsync(ws, 0, sizeof(int), s);
    return (v & NR_FLAG_TIMEOUT) ? NR_ERR_TIMEOUT : NR_OK;
}
