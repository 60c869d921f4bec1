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
// 16 B).  The strips arrive by TMA (activations are stored in 8-channel planes
// so that a strip's K chunk is one contiguous block); a CTA walks along y so
// that each staged input row serves the three output rows that read it, and a
// producer warp, an MMA warp and two groups of epilogue warps overlap staging,
// MMAs and stores (conv32_walk_kernel).  Weights of all 27 taps stay in shared
// memory.  1-channel inputs gather the 27 neighbours into one K = 32 row
// instead.  Weight gradients are GEMMs over voxels on the tensor cores
// (wgrad_tc_kernel), ending in a fixed-order reduction of per-CTA partials.
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

// ---- strip staging shared by the convolution and the weight gradient ------
// A strip is 130 input rows (x0 - 1 .. x0 + 128) of one (patch, z, y) row in
// four planes of 8 channels, each plane a K-major core-matrix column block
// (rows 16 bytes apart) for the MMAs.
constexpr int PLANE = 2176;                           // one K-chunk plane: 130 rows x 16 B, 128-B aligned
constexpr int TSTRIP = KCH * PLANE;                   // 8704 bytes per staged strip
constexpr uint32_t STRIP_TX = (uint32_t)KCH * SROWS * 16;  // bytes the four boxes deliver

// One strip (130 rows x 4 K-chunk planes, plane stride `pstride`) of row
// `row` from x0 - 1 by TMA.  The activation tensor is mapped as (2 nx 8-byte
// units, 4 K chunks, R rows), so one plane is one contiguous run; it is loaded
// as two boxes, rows 0-63 (map lo, 128 units) and rows 64-129 (map hi, 132
// units), both 128-byte aligned in shared memory.  Out-of-range units (x < 0,
// x >= nx, row < 0) arrive as zeros; 4 x 2080 bytes complete on `bar`.
__device__ __forceinline__ void load_strip(uint8_t* dst, int pstride, const CUtensorMap* lo,
                                           const CUtensorMap* hi, int x0, int row, uint64_t* bar) {
    const int u0 = 2 * (x0 - 1);
#pragma unroll
    for (int kc = 0; kc < KCH; kc++) {
        tma_load_3d(dst + kc * pstride, lo, u0, kc, row, bar);
        tma_load_3d(dst + kc * pstride + 1024, hi, u0 + 128, kc, row, bar);
    }
}

// Named barriers over the n threads of a group of warps (id >= 1; id 0 is
// __syncthreads).  group_all is also a vote: true when v is true in every
// thread.  Every warp of the group must reach each of them the same number of
// times; callers take their decisions to stop from group_all, so that no warp
// leaves while the others wait.
__device__ __forceinline__ bool group_all(bool v, int id, int n) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.and.pred p, %2, %3, q;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "r"(n)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void group_sync(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// A bounded wait that also gives up once the block has aborted.
__device__ __forceinline__ bool wait_live(uint64_t* bar, uint32_t parity, volatile int* abort) {
    for (int round = 0; round < WAIT_LIMIT / 1024; round++) {
        if (tc::mbar_wait(bar, parity, 1024)) return true;
        if (*abort) return false;
    }
    return false;
}

// ---- conv32: TMA + tcgen05, walking along y -----------------------------------
// 32-channel input, NOUT = 32 (hidden / input gradient) or 16 (the last layer,
// output channel 0 real) outputs; weights: 27 packed taps of NOUT x 32; one
// output tile (128 x of a row) per TMEM accumulator, staging shared between
// neighbouring output rows.  A work item is a run of up to L output
// rows y0 .. y0 + L - 1 of one column (patch b, plane z, x tile); its tiles
// read the row-sets Y = y0 - 1 .. y0 + L, a row-set being the strips of input
// row Y in planes z - 1, z, z + 1.  Each row-set is loaded once into a ring of
// W_R slots and serves the up to three tiles that read it, so an input row is
// staged about (L + 2) / L times per plane instead of nine.  A strip outside
// the patch is loaded from row -1 (zero-filled), so that every tile issues the
// same 54 MMAs, with descriptors formed as base + compile-time offset.
//   warp 8 (one lane)  producer: row-sets in order into the ring ("full"),
//                      after the slot's previous row-set was released;
//   warp 9 (one lane)  MMA issuer: per tile the row-sets i, i + 1, i + 2 of
//                      the item, 6 MMAs per valid strip, into accumulator
//                      lt & 1; row-set i is released (tcgen05.commit to its
//                      "empty") right after its MMAs -- its last use -- and
//                      the item's last two after its last tile;
//   warps 0-3, 4-7     two epilogue groups, group g for the tiles lt with
//                      lt & 1 == g, so that two epilogues run at once.
// One CTA per SM (the ring and all 27 taps' weights).  Every wait is bounded
// and also gives up once another role has aborted; a role that gives up flags
// NR_FLAG_TIMEOUT and aborts the block.  Before TMEM is released the issuer's
// MMAs are drained, and the producer waits for every copy it issued.
// Measured against the previous form (nine strips per tile, two CTAs per SM):
// L2 traffic falls from 67 % to 8 % of its throughput and the network's
// forward pass on the clinical volume from 22.6-23.0 to 22.5 ms -- the MMAs'
// front end (sm__pipe_tc 57 % with the math at 14 %: an N = 32 MMA reads 5 KB
// of operands for 65 K MACs) paces both.
constexpr int W_R = 6;                                 // row-set slots
constexpr int W_SET = 3 * TSTRIP;                      // 26112 bytes
constexpr int W_THREADS = 320;

struct WalkCtl {
    uint64_t full[W_R], empty[W_R], accf[2], acce[2], drain;
    uint32_t tslot;
    int abort;
};

struct WalkPlan {
    int L, nchunk;
    int tw;  // outputs per tile along x
    int64_t nitems;
};

// Column (b, z, x0) and rows y0 .. y0 + ly - 1 of item it.
__device__ __forceinline__ void item_pos(const Dims& d, const WalkPlan& w, int64_t it, int& b,
                                         int& z, int& x0, int& y0, int& ly) {
    const int xt = (d.nx + w.tw - 1) / w.tw;
    int64_t col = it / w.nchunk;
    const int ch = (int)(it - col * w.nchunk);
    x0 = (int)(col % xt) * w.tw;
    col /= xt;
    z = (int)(col % d.nz);
    b = (int)(col / d.nz);
    y0 = ch * w.L;
    ly = min(w.L, d.ny - y0);
}

// Epilogue of output row `row` (one (patch, z, y) row), voxel x.
template <int EPI>
__device__ __forceinline__ void epilogue_rx(const uint32_t* acc, int64_t row, int x, int nx,
                                            const float* __restrict__ bias, void* out,
                                            const __nv_bfloat16* __restrict__ mask) {
    if (EPI == EPI_RESID) {
        ((float*)out)[row * nx + x] = __uint_as_float(acc[0]) + bias[0];
        return;
    }
    const int64_t o0 = row * KCH * (int64_t)nx * 8 + (int64_t)x * 8;  // chunk q at o0 + q nx 8
    __align__(16) __nv_bfloat16 o[C];
    if (EPI == EPI_RELU) {
        // the bias in FP32, then BF16 pairs and the ReLU on the pairs (rounding
        // is monotone, so max(round(v), 0) = round(max(v, 0)) up to a zero's sign)
        const __nv_bfloat162 zero2 = __float2bfloat162_rn(0.f);
#pragma unroll
        for (int c = 0; c < C; c += 2)
            ((__nv_bfloat162*)o)[c / 2] =
                __hmax2(__floats2bfloat162_rn(__uint_as_float(acc[c]) + bias[c],
                                              __uint_as_float(acc[c + 1]) + bias[c + 1]),
                        zero2);
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

template <int NOUT, int EPI>
__global__ void __launch_bounds__(W_THREADS, 1) conv32_walk_kernel(
    Dims d, WalkPlan wp, const __grid_constant__ CUtensorMap amap,
    const __grid_constant__ CUtensorMap amap_hi, const __nv_bfloat16* __restrict__ wpk,
    const float* __restrict__ bias, void* out, const __nv_bfloat16* __restrict__ mask,
    int* status) {
    constexpr int WBYTES = 27 * NOUT * C * 2;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* ring = smem;
    uint8_t* sW = smem + W_R * W_SET;
    WalkCtl* K = (WalkCtl*)(sW + WBYTES);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int k = tid; k < WBYTES / 16; k += W_THREADS)
        ((uint4*)sW)[k] = __ldg((const uint4*)wpk + k);
    if (tid == 0) {
        for (int s = 0; s < W_R; s++) {
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
    volatile int* abort = &K->abort;
    auto fail = [&]() {
        if (!*abort) atomicOr(status, NR_FLAG_TIMEOUT);
        *abort = 1;
        __threadfence_block();
    };
    auto strip_ok = [&](int zz, int yy) { return zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny; };
    if (warp == 8) {
        if (lane == 0) {
            // producer
            int64_t G = 0, issued = 0;
            bool stop = false;
            for (int64_t it = blockIdx.x; it < wp.nitems && !stop && !*abort; it += gridDim.x) {
                int b, z, x0, y0, ly;
                item_pos(d, wp, it, b, z, x0, y0, ly);
                for (int j = 0; j < ly + 2; j++, G++) {
                    const int s = (int)(G % W_R);
                    if (G >= W_R &&
                        !wait_live(&K->empty[s], (uint32_t)((G / W_R - 1) & 1), abort)) {
                        fail();
                        stop = true;
                        break;
                    }
                    const int Y = y0 - 1 + j;
                    mbar_arrive_tx(&K->full[s], 3 * STRIP_TX);
                    for (int dz = 0; dz < 3; dz++)
                        load_strip(ring + s * W_SET + dz * TSTRIP, PLANE, &amap, &amap_hi, x0,
                                   strip_ok(z + dz - 1, Y) ? (b * d.nz + z + dz - 1) * d.ny + Y : -1,
                                   &K->full[s]);
                    issued = G + 1;
                }
            }
            // no copy may be in flight when the block exits
            for (int64_t k = issued > W_R ? issued - W_R : 0; k < issued; k++) {
                uint64_t* bar = &K->full[k % W_R];
                if (!tc::mbar_wait(bar, (uint32_t)((k / W_R) & 1), WAIT_LIMIT))
                    tc::mbar_wait(bar, (uint32_t)((k / W_R) & 1), WAIT_LIMIT);
            }
        }
    } else if (warp == 9) {
        if (lane == 0) {
            // MMA issuer
            constexpr uint32_t idesc = tc::idesc_bf16(TM, NOUT);
            const uint64_t ad0 = tc::sdesc(tc::smem_u32(ring), PLANE, 128);
            const uint64_t bd0 = tc::sdesc(tc::smem_u32(sW), 128, 512);
            int64_t G = 0;
            int lt = 0;
            bool stop = false;
            for (int64_t it = blockIdx.x; it < wp.nitems && !stop && !*abort; it += gridDim.x) {
                int b, z, x0, y0, ly;
                item_pos(d, wp, it, b, z, x0, y0, ly);
                for (int i = 0; i < ly && !stop; i++, lt++) {
                    const int a = lt & 1;
                    if (lt >= 2 &&
                        !wait_live(&K->acce[a], (uint32_t)(((lt >> 1) - 1) & 1), abort)) {
                        fail();
                        stop = true;
                        break;
                    }
                    tc::fence_after();
                    const uint32_t dacc = tmem + (uint32_t)(a * 32);
#pragma unroll
                    for (int dy = 0; dy < 3; dy++) {
                        const int64_t gs = G + i + dy;
                        const int s = (int)(gs % W_R);
                        if ((i == 0 || dy == 2) &&
                            !wait_live(&K->full[s], (uint32_t)((gs / W_R) & 1), abort)) {
                            fail();
                            stop = true;
                            break;
                        }
                        tc::fence_after();
                        // descriptors are linear in the address: base + offset / 16
                        const uint64_t adr = ad0 + (uint64_t)((s * W_SET) >> 4);
#pragma unroll
                        for (int dz = 0; dz < 3; dz++)
#pragma unroll
                            for (int dx = 0; dx < 3; dx++)
#pragma unroll
                                for (int j = 0; j < 2; j++) {
                                    const int tap = dz * 9 + dy * 3 + dx;
                                    tc::mma_bf16(
                                        dacc,
                                        adr + (uint64_t)((dz * TSTRIP + dx * 16 + j * 2 * PLANE) >> 4),
                                        bd0 + (uint64_t)((tap * NOUT * C * 2 + j * 256) >> 4), idesc,
                                        (dy | dz | dx | j) ? 1u : 0u);
                                }
                        // row-set i is not read after this tile; the last tile
                        // of the item also frees row-sets ly and ly + 1
                        if (dy == 0 || i == ly - 1) tc::commit(&K->empty[s]);
                    }
                    if (stop) break;
                    tc::commit(&K->accf[a]);
                }
                G += ly + 2;
            }
        }
    } else {
        // epilogue group g = warp / 4: TMEM lanes 32 (warp % 4) .. + 31 of the
        // tiles lt with lt & 1 == g.  Test hook: the workspace's second status
        // word k + 1 > 0 makes the wait for this CTA's tile k report giving up
        // once it has in fact succeeded.
        const int g = warp >> 2, wq = warp & 3;
        const int force_at = status[1] - 1;
        int lt = 0;
        bool stop = false;
        for (int64_t it = blockIdx.x; it < wp.nitems && !stop; it += gridDim.x) {
            int b, z, x0, y0, ly;
            item_pos(d, wp, it, b, z, x0, y0, ly);
            for (int i = 0; i < ly; i++, lt++) {
                if ((lt & 1) != g) continue;
                bool got = wait_live(&K->accf[g], (uint32_t)((lt >> 1) & 1), abort);
                if (lt == force_at) got = false;
                if (!got) {
                    if (lane == 0) fail();
                    stop = true;
                    break;
                }
                tc::fence_after();
                uint32_t acc[32];
                tc::ld32(tmem, (uint32_t)(wq * 32), (uint32_t)(g * 32), acc);
                tc::fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&K->acce[g]);
                const int x = x0 + wq * 32 + lane;
                if (x < d.nx)
                    epilogue_rx<EPI>(acc, ((int64_t)b * d.nz + z) * d.ny + y0 + i, x, d.nx, bias,
                                     out, mask);
            }
        }
    }
    // drain: every MMA issued has completed before TMEM is released
    __syncthreads();
    if (warp == 9 && lane == 0) tc::commit(&K->drain);
    if (!tc::mbar_wait(&K->drain, 0, WAIT_LIMIT)) tc::mbar_wait(&K->drain, 0, WAIT_LIMIT);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// ---- conv32 with the three dx taps in one MMA -------------------------------
// The walk of conv32_walk_kernel with N = 3 NOUT: the weights of the three dx
// taps of a strip are adjacent in the packed buffer (512-byte row groups), so
// one MMA over the unshifted strip (A rows r = input x0 - 1 + r) computes
// D[r][(dx, o)] = sum_i a[x0 - 1 + r][i] W[dz][dy][dx][o][i] for all three dx:
// 18 MMAs per tile instead of 54, and each A row is fetched once per strip
// instead of three times.  Output x0 - 1 + r (r = 1 .. 126: 126 outputs per
// tile, tiles 126 apart) is D[r - 1][dx 0] + D[r][dx 1] + D[r + 1][dx 2]: the
// dx = 0 and dx = 2 columns are moved one TMEM lane by warp shuffles, and
// across the four warps' lane quarters through shared memory (each warp
// publishes lane 31's dx-0 and lane 0's dx-2 columns, double-buffered by
// tile; a named barrier per epilogue group orders the exchange, the group
// having voted on the accumulator wait first, so that its warps stop
// together or not at all).  TMEM: two accumulators of 3 NOUT columns (at 0 and 128).
constexpr int W3_TW = TM - 2;  // 126 outputs per tile
constexpr int W3_NG = 4;       // epilogue groups = TMEM accumulators
constexpr int W3_THREADS = 32 * (4 * W3_NG + 2);

struct W3Ctl {
    uint64_t full[W_R], empty[W_R], accf[W3_NG], acce[W3_NG], drain;
    uint32_t tslot;
    int abort;
    float xb[W3_NG][2][4][2][C];  // [group][tile parity][warp][lane 31 dx 0 | lane 0 dx 2][o]
};

template <int NOUT, int EPI>
__global__ void __launch_bounds__(W3_THREADS, 1) conv32_w3_kernel(
    Dims d, WalkPlan wp, const __grid_constant__ CUtensorMap amap,
    const __grid_constant__ CUtensorMap amap_hi, const __nv_bfloat16* __restrict__ wpk,
    const float* __restrict__ bias, void* out, const __nv_bfloat16* __restrict__ mask,
    int* status) {
    constexpr int WBYTES = 27 * NOUT * C * 2;
    constexpr int NO = EPI == EPI_RESID ? 1 : NOUT;  // output channels the epilogue needs
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* ring = smem;
    uint8_t* sW = smem + W_R * W_SET;
    W3Ctl* K = (W3Ctl*)(sW + WBYTES);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int k = tid; k < WBYTES / 16; k += W3_THREADS)
        ((uint4*)sW)[k] = __ldg((const uint4*)wpk + k);
    if (tid == 0) {
        for (int s = 0; s < W_R; s++) {
            tc::mbar_init(&K->full[s], 1);
            tc::mbar_init(&K->empty[s], 1);
        }
        for (int a = 0; a < W3_NG; a++) {
            tc::mbar_init(&K->accf[a], 1);
            tc::mbar_init(&K->acce[a], 4);
        }
        tc::mbar_init(&K->drain, 1);
        K->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::tmem_alloc(&K->tslot, 512);
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = K->tslot;
    volatile int* abort = &K->abort;
    auto fail = [&]() {
        if (!*abort) atomicOr(status, NR_FLAG_TIMEOUT);
        *abort = 1;
        __threadfence_block();
    };
    auto strip_ok = [&](int zz, int yy) { return zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny; };
    if (warp == 4 * W3_NG) {
        if (lane == 0) {
            // producer (as in conv32_walk_kernel)
            int64_t G = 0, issued = 0;
            bool stop = false;
            for (int64_t it = blockIdx.x; it < wp.nitems && !stop && !*abort; it += gridDim.x) {
                int b, z, x0, y0, ly;
                item_pos(d, wp, it, b, z, x0, y0, ly);
                for (int j = 0; j < ly + 2; j++, G++) {
                    const int s = (int)(G % W_R);
                    if (G >= W_R &&
                        !wait_live(&K->empty[s], (uint32_t)((G / W_R - 1) & 1), abort)) {
                        fail();
                        stop = true;
                        break;
                    }
                    const int Y = y0 - 1 + j;
                    mbar_arrive_tx(&K->full[s], 3 * STRIP_TX);
                    for (int dz = 0; dz < 3; dz++)
                        load_strip(ring + s * W_SET + dz * TSTRIP, PLANE, &amap, &amap_hi, x0,
                                   strip_ok(z + dz - 1, Y) ? (b * d.nz + z + dz - 1) * d.ny + Y : -1,
                                   &K->full[s]);
                    issued = G + 1;
                }
            }
            for (int64_t k = issued > W_R ? issued - W_R : 0; k < issued; k++) {
                uint64_t* bar = &K->full[k % W_R];
                if (!tc::mbar_wait(bar, (uint32_t)((k / W_R) & 1), WAIT_LIMIT))
                    tc::mbar_wait(bar, (uint32_t)((k / W_R) & 1), WAIT_LIMIT);
            }
        }
    } else if (warp == 4 * W3_NG + 1) {
        if (lane == 0) {
            // MMA issuer: per strip (dz, dy) two MMAs of K = 16, N = 3 NOUT
            constexpr uint32_t idesc = tc::idesc_bf16(TM, 3 * NOUT);
            const uint64_t ad0 = tc::sdesc(tc::smem_u32(ring), PLANE, 128);
            const uint64_t bd0 = tc::sdesc(tc::smem_u32(sW), 128, 512);
            int64_t G = 0;
            int lt = 0;
            bool stop = false;
            for (int64_t it = blockIdx.x; it < wp.nitems && !stop && !*abort; it += gridDim.x) {
                int b, z, x0, y0, ly;
                item_pos(d, wp, it, b, z, x0, y0, ly);
                for (int i = 0; i < ly && !stop; i++, lt++) {
                    const int a = lt % W3_NG;
                    if (lt >= W3_NG &&
                        !wait_live(&K->acce[a], (uint32_t)((lt / W3_NG - 1) & 1), abort)) {
                        fail();
                        stop = true;
                        break;
                    }
                    tc::fence_after();
                    const uint32_t dacc = tmem + (uint32_t)(a * 128);
#pragma unroll
                    for (int dy = 0; dy < 3; dy++) {
                        const int64_t gs = G + i + dy;
                        const int s = (int)(gs % W_R);
                        if ((i == 0 || dy == 2) &&
                            !wait_live(&K->full[s], (uint32_t)((gs / W_R) & 1), abort)) {
                            fail();
                            stop = true;
                            break;
                        }
                        tc::fence_after();
                        const uint64_t adr = ad0 + (uint64_t)((s * W_SET) >> 4);
#pragma unroll
                        for (int dz = 0; dz < 3; dz++)
#pragma unroll
                            for (int j = 0; j < 2; j++)
                                tc::mma_bf16(
                                    dacc, adr + (uint64_t)((dz * TSTRIP + j * 2 * PLANE) >> 4),
                                    bd0 + (uint64_t)(((dz * 9 + dy * 3) * NOUT * C * 2 + j * 256) >> 4),
                                    idesc, (dy | dz | j) ? 1u : 0u);
                        if (dy == 0 || i == ly - 1) tc::commit(&K->empty[s]);
                    }
                    if (stop) break;
                    tc::commit(&K->accf[a]);
                }
                G += ly + 2;
            }
        }
    } else {
        // epilogue group g = warp / 4 (tiles lt with lt % W3_NG == g); TMEM lane
        // 32 wq + lane = tile row r.  Test hook as in conv32_walk_kernel.
        const int g = warp >> 2, wq = warp & 3;
        const int force_at = status[1] - 1;
        int lt = 0, kg = 0;
        bool stop = false;
        for (int64_t it = blockIdx.x; it < wp.nitems && !stop; it += gridDim.x) {
            int b, z, x0, y0, ly;
            item_pos(d, wp, it, b, z, x0, y0, ly);
            for (int i = 0; i < ly; i++, lt++) {
                if (lt % W3_NG != g) continue;
                bool got = wait_live(&K->accf[g], (uint32_t)((lt / W3_NG) & 1), abort);
                if (lt == force_at) got = false;
                if (!group_all(got, 1 + g, 128)) {  // the group stops together
                    if (lane == 0) fail();
                    stop = true;
                    break;
                }
                tc::fence_after();
                // columns: dx 0 at col, dx 1 at col + NOUT, dx 2 at col + 2 NOUT.
                // First publish the lane-quarter edges (lane 31's dx 0, lane 0's
                // dx 2), then, after the group barrier, read the columns again
                // into a running sum: at most 64 accumulator values live.
                const uint32_t col = (uint32_t)(g * 128), l0 = (uint32_t)(wq * 32);
                float* xb = &K->xb[g][kg & 1][0][0][0];
                uint32_t c[32];
                tc::ld32(tmem, l0, col, c);
                if (lane == 31)
                    for (int o = 0; o < NO; o++) xb[(wq * 2 + 0) * C + o] = __uint_as_float(c[o]);
                tc::ld32(tmem, l0, col + 2 * NOUT, c);
                if (lane == 0)
                    for (int o = 0; o < NO; o++) xb[(wq * 2 + 1) * C + o] = __uint_as_float(c[o]);
                group_sync(1 + g, 128);
                kg++;
                float sum[NO];
                tc::ld32(tmem, l0, col, c);
#pragma unroll
                for (int o = 0; o < NO; o++) {
                    float up = __shfl_up_sync(0xffffffffu, __uint_as_float(c[o]), 1);
                    if (lane == 0) up = wq > 0 ? xb[((wq - 1) * 2 + 0) * C + o] : 0.f;
                    sum[o] = up;
                }
                tc::ld32(tmem, l0, col + NOUT, c);
#pragma unroll
                for (int o = 0; o < NO; o++) sum[o] = sum[o] + __uint_as_float(c[o]);
                tc::ld32(tmem, l0, col + 2 * NOUT, c);
                tc::fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&K->acce[g]);
                uint32_t acc[32];
#pragma unroll
                for (int o = 0; o < NO; o++) {
                    float dn = __shfl_down_sync(0xffffffffu, __uint_as_float(c[o]), 1);
                    if (lane == 31) dn = wq < 3 ? xb[((wq + 1) * 2 + 1) * C + o] : 0.f;
                    acc[o] = __float_as_uint(sum[o] + dn);
                }
                const int r = wq * 32 + lane, x = x0 - 1 + r;
                if (r >= 1 && r <= W3_TW && x < d.nx)
                    epilogue_rx<EPI>(acc, ((int64_t)b * d.nz + z) * d.ny + y0 + i, x, d.nx, bias,
                                     out, mask);
            }
        }
    }
    __syncthreads();
    if (warp == 4 * W3_NG + 1 && lane == 0) tc::commit(&K->drain);
    if (!tc::mbar_wait(&K->drain, 0, WAIT_LIMIT)) tc::mbar_wait(&K->drain, 0, WAIT_LIMIT);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// ---- the 32 -> 1 layer in two passes -----------------------------------------
// f[v] = b + sum over taps of W[tap] . a[v + off(tap)], regrouped by the tap's
// (dz, dy).  Pass 1 (last_rows_kernel), per input row u of the volume:
//     q[(dz, dy)][u] = sum_dx W[dz][dy][dx] . a[u + (dx - 1, 0, 0)]
// as three MMAs (one per dx: the row's strip at a 16-byte offset) of N = 16
// (rows (dz, dy), 9 used) and K = 32 per 128 voxels -- one strip per tile
// against the convolution's nine, and no walk.  Pass 2 (last_sum_kernel):
//     f[v] = b + sum_{(dz, dy)} q[(dz, dy)][v + (0, dy - 1, dz - 1)]
// (zero outside the patch), nine coalesced loads in a fixed order.  Pass 1:
// a producer lane loads the strips into a ring of LR_STAGE stages, an issuer
// lane runs the MMAs into one of two TMEM accumulators, four epilogue warps
// store the nine planes of q; waits bounded as in conv32_walk_kernel.
constexpr int LR_STAGE = 6;
constexpr int LR_THREADS = 192;

struct LastCtl {
    uint64_t full[LR_STAGE], empty[LR_STAGE], accf[2], acce[2], drain;
    uint32_t tslot;
    int abort;
};

__global__ void __launch_bounds__(LR_THREADS) last_rows_kernel(
    Dims d, const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap amap_hi,
    const __nv_bfloat16* __restrict__ wpk, float* __restrict__ q, int* status) {
    constexpr int WBYTES = 3 * 16 * C * 2;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* ring = smem;
    uint8_t* sW = smem + LR_STAGE * TSTRIP;
    LastCtl* K = (LastCtl*)(sW + WBYTES);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int k = tid; k < WBYTES / 16; k += LR_THREADS)
        ((uint4*)sW)[k] = __ldg((const uint4*)wpk + k);
    if (tid == 0) {
        for (int s = 0; s < LR_STAGE; s++) {
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
    const int64_t V = nvox(d);
    volatile int* abort = &K->abort;
    auto fail = [&]() {
        if (!*abort) atomicOr(status, NR_FLAG_TIMEOUT);
        *abort = 1;
        __threadfence_block();
    };
    if (warp == 4) {
        if (lane == 0) {
            // producer
            int64_t lt = 0, issued = 0;
            for (int64_t t = blockIdx.x; t < nt && !*abort; t += gridDim.x, lt++) {
                const int s = (int)(lt % LR_STAGE);
                if (lt >= LR_STAGE &&
                    !wait_live(&K->empty[s], (uint32_t)((lt / LR_STAGE - 1) & 1), abort)) {
                    fail();
                    break;
                }
                int b, z, y, x0;
                tile_pos(d, t, b, z, y, x0);
                mbar_arrive_tx(&K->full[s], STRIP_TX);
                load_strip(ring + s * TSTRIP, PLANE, &amap, &amap_hi, x0, (b * d.nz + z) * d.ny + y,
                           &K->full[s]);
                issued = lt + 1;
            }
            for (int64_t k = issued > LR_STAGE ? issued - LR_STAGE : 0; k < issued; k++) {
                uint64_t* bar = &K->full[k % LR_STAGE];
                if (!tc::mbar_wait(bar, (uint32_t)((k / LR_STAGE) & 1), WAIT_LIMIT))
                    tc::mbar_wait(bar, (uint32_t)((k / LR_STAGE) & 1), WAIT_LIMIT);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            // MMA issuer: per dx, the strip at offset dx rows against its 16 x 32 block
            constexpr uint32_t idesc = tc::idesc_bf16(TM, 16);
            const uint64_t ad0 = tc::sdesc(tc::smem_u32(ring), PLANE, 128);
            const uint64_t bd0 = tc::sdesc(tc::smem_u32(sW), 128, 512);
            int64_t lt = 0;
            for (int64_t t = blockIdx.x; t < nt && !*abort; t += gridDim.x, lt++) {
                const int a = (int)(lt & 1), s = (int)(lt % LR_STAGE);
                if (lt >= 2 && !wait_live(&K->acce[a], (uint32_t)(((lt >> 1) - 1) & 1), abort)) {
                    fail();
                    break;
                }
                if (!wait_live(&K->full[s], (uint32_t)((lt / LR_STAGE) & 1), abort)) {
                    fail();
                    break;
                }
                tc::fence_after();
                const uint64_t adr = ad0 + (uint64_t)((s * TSTRIP) >> 4);
#pragma unroll
                for (int dx = 0; dx < 3; dx++)
#pragma unroll
                    for (int j = 0; j < 2; j++)
                        tc::mma_bf16(tmem + (uint32_t)(a * 32),
                                     adr + (uint64_t)((dx * 16 + j * 2 * PLANE) >> 4),
                                     bd0 + (uint64_t)((dx * 16 * C * 2 + j * 256) >> 4), idesc,
                                     (dx | j) ? 1u : 0u);
                tc::commit(&K->empty[s]);
                tc::commit(&K->accf[a]);
            }
        }
    } else {
        // epilogue warps 0-3: row 32 warp + lane of each tile.  Test hook: the
        // workspace's second status word k + 1 > 0 makes the wait for this
        // CTA's tile k report giving up once it has in fact succeeded.
        const int force_at = status[1] - 1;
        int64_t lt = 0;
        for (int64_t t = blockIdx.x; t < nt; t += gridDim.x, lt++) {
            const int a = (int)(lt & 1);
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
            int b, z, y, x0;
            tile_pos(d, t, b, z, y, x0);
            const int x = x0 + warp * 32 + lane;
            if (x < d.nx) {
                const int64_t v = (((int64_t)b * d.nz + z) * d.ny + y) * d.nx + x;
#pragma unroll
                for (int n = 0; n < 9; n++) q[n * V + v] = __uint_as_float(acc[n]);
            }
        }
    }
    __syncthreads();
    if (warp == 5 && lane == 0) tc::commit(&K->drain);
    if (!tc::mbar_wait(&K->drain, 0, WAIT_LIMIT)) tc::mbar_wait(&K->drain, 0, WAIT_LIMIT);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// Pass 2: grid (row of the stacked volume, block of 256 x VEC); VEC = 4 when
// rows are 16-byte aligned (nx % 4 == 0): four x per thread in float4 loads.
template <int VEC>
__global__ void __launch_bounds__(256) last_sum_kernel(Dims d, const float* __restrict__ q,
                                                       const float* __restrict__ bias,
                                                       float* __restrict__ f) {
    const int64_t row = blockIdx.x;
    const int x = (blockIdx.y * 256 + threadIdx.x) * VEC;
    if (x >= d.nx) return;
    const int y = (int)(row % d.ny), z = (int)((row / d.ny) % d.nz);
    const int64_t b = row / ((int64_t)d.ny * d.nz);
    const int64_t V = nvox(d);
    if (VEC == 4) {
        float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int n = 0; n < 9; n++) {
            const int zz = z + n / 3 - 1, yy = y + n % 3 - 1;
            if (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny) {
                const float4 v =
                    __ldg((const float4*)(q + n * V + ((b * d.nz + zz) * d.ny + yy) * d.nx + x));
                sum.x += v.x;
                sum.y += v.y;
                sum.z += v.z;
                sum.w += v.w;
            }
        }
        const float b0 = bias[0];
        *(float4*)(f + row * d.nx + x) =
            make_float4(sum.x + b0, sum.y + b0, sum.z + b0, sum.w + b0);
    } else {
        float sum = 0.f;
#pragma unroll
        for (int n = 0; n < 9; n++) {
            const int zz = z + n / 3 - 1, yy = y + n % 3 - 1;
            if (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny)
                sum += __ldg(q + n * V + ((b * d.nz + zz) * d.ny + yy) * d.nx + x);
        }
        f[row * d.nx + x] = sum + bias[0];
    }
}

// 1-channel input conv (the first layer, and the back projection of the last
// layer's gradient): each output row gathers its 27 neighbours (zero outside
// its patch) x scale into one K = 32 row.  Weights: one packed 32 x 32 tile.
template <int EPI>
__global__ void __launch_bounds__(128) conv1_kernel(Dims d, WalkPlan wp, const float* __restrict__ in,
                                                    float scale,
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
    int ntile = 0;
    int ncommit = 0;
    bool ok = true;
    const int force_at = status[1] - 1;  // test hook, as in conv32_walk_kernel
    // Tiles in runs of rows along y (the items of conv32_walk_kernel), so
    // that consecutive tiles of a CTA share six of their nine input rows.
    struct Pos {
        int64_t it;
        int i, b, z, y0, ly, x0;
    };
    auto first = [&](int64_t it, Pos& p) {
        p.it = it;
        p.i = 0;
        if (it < wp.nitems) item_pos(d, wp, it, p.b, p.z, p.x0, p.y0, p.ly);
    };
    auto advance = [&](Pos& p) {
        if (++p.i >= p.ly) first(p.it + gridDim.x, p);
    };
    // the 27 neighbours of this thread's voxel in a tile (zero outside the
    // patch), loaded one tile ahead so that their latency overlaps the
    // previous tile's MMAs and epilogue
    // The nine rows' bases and validity and the three x offsets' validity
    // are formed once per tile; each tap is then one predicated load.
    float nb[27];
    auto gather = [&](const Pos& p) {
        const int b = p.b, z = p.z, y = p.y0 + p.i;
        const int x = p.x0 + tid;
        const bool xv[3] = {x >= 1 && x - 1 < d.nx, x < d.nx, x + 1 < d.nx};
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const int zz = z + q / 3 - 1, yy = y + q % 3 - 1;
            const bool rv = zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny;
            const float* row = in + (((int64_t)b * d.nz + (rv ? zz : z)) * d.ny + (rv ? yy : y)) * d.nx;
#pragma unroll
            for (int dx = 0; dx < 3; dx++)
                nb[3 * q + dx] = (rv && xv[dx]) ? __ldg(row + x + dx - 1) : 0.f;
        }
    };
    Pos cur, nxt;
    first(blockIdx.x, cur);
    if (cur.it < wp.nitems) gather(cur);
    for (; cur.it < wp.nitems; cur = nxt) {
        nxt = cur;
        advance(nxt);
        const int b = cur.b, z = cur.z, y = cur.y0 + cur.i, x0 = cur.x0;
        const int x = x0 + tid;
        __align__(16) __nv_bfloat162 row[16];
#pragma unroll
        for (int k = 0; k < 16; k++)
            row[k] = __floats2bfloat162_rn(2 * k < 27 ? nb[2 * k] * scale : 0.f,
                                           2 * k + 1 < 27 ? nb[2 * k + 1] * scale : 0.f);
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
        if (nxt.it < wp.nitems) gather(nxt);
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
        if (x < d.nx) epilogue_rx<EPI>(acc, ((int64_t)b * d.nz + z) * d.ny + y, x, d.nx, bias, out, mask);
        tc::fence_before();
        __syncthreads();
    }
    if (tid == 0) tc::commit(&bars[0]);  // drain: every MMA issued completes before TMEM goes
    if (!tc::mbar_wait(&bars[0], (uint32_t)(ncommit & 1), WAIT_LIMIT))
        tc::mbar_wait(&bars[0], (uint32_t)(ncommit & 1), WAIT_LIMIT);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 32);
}

// ---------------------------------------------------------------------------
// Weight gradients on the tensor cores.  dW[tap][o][i] = sum_v g[v][o]
// in[v + off(tap)][i] over the stacked patches (zero outside each patch) and
// db[o] = sum_v g[v][o]: per layer one GEMM with the voxels as K, in K blocks
// of one tile (128 consecutive x of a (patch, z, y) row).
//
// The activations' plane layout makes staged strips operands as they land: a
// strip plane is [x][8 channels], i.e. MN-major core matrices (8 channels x 8
// consecutive x in 16-byte rows), and strips staged one after another sit at
// one uniform plane stride, so several strips form one operand whose rows are
// (strip, channel), and a shift along x is a 16-byte start offset.
// This kernel serves the 1-channel layers (the 32 -> 32 ones walk along y in
// wgrad_walk_kernel, below):
//   WG_LAST  (32 -> 1)   A = four input strips (rows (strip, i)) at the tap's
//                        x shift: blocks {0-3}, {4-7}, {5-8} (of the last only
//                        strip 8's rows are kept) x dx = 9 MMA blocks; B = the
//                        FP32 gradient of the one output split as hi + lo BF16
//                        (rows 0, 1 of an N = 16 K-major operand): dW = column
//                        0 + column 1.
//   WG_FIRST (1 -> 32)   A = the FP32 input u = s x at the 27 shifts split as
//                        hi (rows 0-26) + lo (rows 32-58) of a K-major M = 128
//                        operand; B = the gradient strip.
// The split keeps the FP32 operand to 2^-17 relative: hi = bf16(u), lo =
// bf16(u - hi), and the products of BF16 values are exact in the FP32
// accumulator.  The bias gradient is summed on the CUDA cores (FP32 per
// thread, then in a fixed order).
//
// Roles (6 warps): warp 0 lane 0 loads each K block's strips by TMA into one
// of two stages (a strip outside the patch in z or y is loaded from row -1,
// i.e. zero-filled); warp 1 lane 0 issues the MMAs and frees the stage by
// tcgen05.commit; warps 2-5 (x - x0 in 32 h .. 32 h + 31 for warp 2 + h) build
// the split operand from global data fetched one block ahead and sum the
// bias.  Every wait is bounded and gives up once another role has aborted; a
// role that gives up flags NR_FLAG_TIMEOUT and aborts the block.  Before TMEM
// is released the issuer's MMAs are drained and the producer waits for every
// copy it issued.  Each CTA writes one partial per weight (row blockIdx.x of
// partial[CTA][28 x weights per tap]); wgrad_reduce_kernel adds the rows in
// order.
enum { WG_LAST = 1, WG_FIRST = 2 };
constexpr int WG_MAXCTA = 256;  // partial slots per weight
constexpr int WG_GROUP = 2048;  // K-major built operand: bytes per 8-row group (16 K chunks)
constexpr int WG_PLANE = 2176;  // staged plane: 130 rows x 16 B, 128-B aligned
constexpr int WG_STRIP = KCH * WG_PLANE;
constexpr int WG_THREADS = 192;
constexpr int WG_WIN = 34;      // WG_FIRST: input window per builder warp and row

struct WgCtl {
    uint64_t tfull[2], bfull[2], empty[2], drain;
    uint32_t tslot;
    int abort;
    float bsum[4][C];
};

template <int MODE>
struct WgCfg {
    // one stage: [input strips 0..8 | gradient strip | built operand]
    static constexpr int NSTRIP = MODE == WG_FIRST ? 0 : 9;
    static constexpr int NCOPY = MODE == WG_FIRST ? 1 : 0;
    static constexpr int NLOAD = NCOPY;
    static constexpr int OFF_G = NSTRIP * WG_STRIP;
    static constexpr int OFF_X = OFF_G + NCOPY * WG_STRIP;
    static constexpr int XBYTES =
        MODE == WG_LAST ? 2 * WG_GROUP : (MODE == WG_FIRST ? 16 * WG_GROUP : 0);
    static constexpr int STAGE = OFF_X + XBYTES;
    static constexpr uint32_t TX = (uint32_t)(NSTRIP + NLOAD) * KCH * SROWS * 16;
    static constexpr int N = MODE == WG_LAST ? 16 : C;
    static constexpr uint32_t NCOL = MODE == WG_FIRST ? 32 : 512;
    // WG_FIRST: each builder warp's window of the input, 9 rows x WG_WIN x
    static constexpr int XS = MODE == WG_FIRST ? 4 * 9 * WG_WIN * 4 : 0;
    static constexpr int SMEM = 2 * STAGE + XS + (int)sizeof(WgCtl);
    // bit 15 / 16: A / B MN-major
    static constexpr uint32_t IDESC = tc::idesc_bf16(TM, N) |
                                      (MODE != WG_FIRST ? 1u << 15 : 0u) |
                                      (MODE != WG_LAST ? 1u << 16 : 0u);
    // arrivals that free a stage: the MMA commit, and the bias warps after
    // reading the gradient strip
    static constexpr int EMPTY_COUNT = MODE == WG_LAST ? 1 : 5;
};

// Stores the BF16 pair hi + lo of u at rows (mh, ml), K index k of a K-major
// built operand (8-row groups WG_GROUP apart, K chunks 128 B apart).
__device__ __forceinline__ void wg_split_store(uint8_t* op, int mh, int ml, int k, float u) {
    const __nv_bfloat16 hi = __float2bfloat16_rn(u);
    const __nv_bfloat16 lo = __float2bfloat16_rn(u - __bfloat162float(hi));
    const int kk = (k >> 3) * 128 + (k & 7) * 2;
    *(__nv_bfloat16*)(op + (mh >> 3) * WG_GROUP + kk + (mh & 7) * 16) = hi;
    *(__nv_bfloat16*)(op + (ml >> 3) * WG_GROUP + kk + (ml & 7) * 16) = lo;
}

// The global data one builder lane needs for the K block of tile t: WG_LAST
// the gradient at x = x0 + 32 h + lane; WG_FIRST its share of the warp's
// window u = s x at x0 - 1 + 32 h + j (j < WG_WIN) of the nine rows.
template <int MODE>
__device__ __forceinline__ void wg_fetch(const Dims& d, int64_t t, int h, int lane,
                                         const float* __restrict__ gvec,
                                         const float* __restrict__ xin, float s, float* r) {
    int b, z, y, x0;
    tile_pos(d, t, b, z, y, x0);
    if (MODE == WG_LAST) {
        const int x = x0 + 32 * h + lane;
        r[0] = x < d.nx ? __ldg(gvec + (((int64_t)b * d.nz + z) * d.ny + y) * d.nx + x) : 0.f;
    } else if (MODE == WG_FIRST) {
#pragma unroll
        for (int k = 0; k < (9 * WG_WIN + 31) / 32; k++) {
            const int e = lane + 32 * k;
            const int q = e / WG_WIN, j = e - q * WG_WIN;
            const int zz = z + q / 3 - 1, yy = y + q % 3 - 1;
            const int xx = x0 - 1 + 32 * h + j;
            r[k] = 0.f;
            if (e < 9 * WG_WIN && zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny && xx >= 0 &&
                xx < d.nx)
                r[k] = __ldg(xin + (((int64_t)b * d.nz + zz) * d.ny + yy) * d.nx + xx) * s;
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(WG_THREADS, 1) wgrad_tc_kernel(
    Dims d, const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap amap_hi,
    const __grid_constant__ CUtensorMap gmap, const __grid_constant__ CUtensorMap gmap_hi,
    const float* __restrict__ gvec, const float* __restrict__ xin, float s,
    float* __restrict__ partial, int* status) {
    using Cfg = WgCfg<MODE>;
    extern __shared__ __align__(1024) uint8_t smem[];
    WgCtl* K = (WgCtl*)(smem + 2 * Cfg::STAGE + Cfg::XS);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // regions the copies and the builders never write stay zero
    constexpr int ZOFF = Cfg::OFF_X;
    constexpr int ZBYTES = Cfg::XBYTES;
    for (int k = tid; k < ZBYTES / 16; k += WG_THREADS) {
        ((uint4*)(smem + ZOFF))[k] = make_uint4(0, 0, 0, 0);
        ((uint4*)(smem + Cfg::STAGE + ZOFF))[k] = make_uint4(0, 0, 0, 0);
    }
    tc::fence_async_smem();
    if (tid == 0) {
        for (int k = 0; k < 2; k++) {
            tc::mbar_init(&K->tfull[k], 1);
            tc::mbar_init(&K->bfull[k], 4);
            tc::mbar_init(&K->empty[k], Cfg::EMPTY_COUNT);
        }
        tc::mbar_init(&K->drain, 1);
        K->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::tmem_alloc(&K->tslot, Cfg::NCOL);
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
    if (warp == 0) {
        if (lane == 0) {
            // producer
            int64_t kb = 0, issued = 0;
            for (int64_t t = blockIdx.x; t < nt && !*abort; t += gridDim.x, kb++) {
                const int sg = (int)(kb & 1);
                if (kb >= 2 &&
                    !wait_live(&K->empty[sg], (uint32_t)(((kb >> 1) - 1) & 1), abort)) {
                    fail();
                    break;
                }
                int b, z, y, x0;
                tile_pos(d, t, b, z, y, x0);
                uint8_t* st = smem + sg * Cfg::STAGE;
                mbar_arrive_tx(&K->tfull[sg], Cfg::TX);
                const int grow = (b * d.nz + z) * d.ny + y;
                // gradient copy c starts at x0 + 1 - c (HID) / x0 - 1 (FIRST)
                for (int c = 0; c < Cfg::NLOAD; c++)
                    load_strip(st + Cfg::OFF_G + c * WG_STRIP, WG_PLANE, &gmap, &gmap_hi,
                               x0, grow, &K->tfull[sg]);
                for (int q = 0; q < Cfg::NSTRIP; q++) {
                    const int zz = z + q / 3 - 1, yy = y + q % 3 - 1;
                    const int row = (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny)
                                        ? (b * d.nz + zz) * d.ny + yy
                                        : -1;
                    load_strip(st + q * WG_STRIP, WG_PLANE, &amap, &amap_hi, x0, row,
                               &K->tfull[sg]);
                }
                issued = kb + 1;
            }
            // no copy may be in flight when the block exits
            for (int64_t k = issued > 2 ? issued - 2 : 0; k < issued; k++) {
                uint64_t* bar = &K->tfull[k & 1];
                if (!tc::mbar_wait(bar, (uint32_t)((k >> 1) & 1), WAIT_LIMIT))
                    tc::mbar_wait(bar, (uint32_t)((k >> 1) & 1), WAIT_LIMIT);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer.  Test hook: the workspace's second status word k + 1
            // > 0 makes the wait for this CTA's K block k report giving up
            // once it has in fact succeeded.
            const int force_at = status[1] - 1;
            int64_t kb = 0;
            for (int64_t t = blockIdx.x; t < nt && !*abort; t += gridDim.x, kb++) {
                const int sg = (int)(kb & 1);
                const uint32_t par = (uint32_t)((kb >> 1) & 1);
                bool got = wait_live(&K->tfull[sg], par, abort);
                if (got) got = wait_live(&K->bfull[sg], par, abort);
                if (kb == force_at) got = false;
                if (!got) {
                    fail();
                    break;
                }
                tc::fence_after();
                const uint32_t sb = tc::smem_u32(smem + sg * Cfg::STAGE);
                if (MODE == WG_FIRST) {
#pragma unroll
                    for (int k = 0; k < TM / 16; k++)
                        tc::mma_bf16(tmem, tc::sdesc(sb + Cfg::OFF_X + k * 256, 128, WG_GROUP),
                                     tc::sdesc(sb + Cfg::OFF_G + 16 + k * 256, 128, WG_PLANE),
                                     Cfg::IDESC, (kb > 0 || k > 0) ? 1u : 0u);
                } else {
                    for (int gi = 0; gi < 3; gi++) {
                        const int g0 = gi == 0 ? 0 : (gi == 1 ? 4 : 5);
#pragma unroll
                        for (int dx = 0; dx < 3; dx++) {
                            const uint32_t dacc = tmem + (uint32_t)((gi * 3 + dx) * 32);
#pragma unroll
                            for (int k = 0; k < TM / 16; k++)
                                tc::mma_bf16(
                                    dacc,
                                    tc::sdesc(sb + g0 * WG_STRIP + dx * 16 + k * 256, 128, WG_PLANE),
                                    tc::sdesc(sb + Cfg::OFF_X + k * 256, 128, WG_GROUP),
                                    Cfg::IDESC, (kb > 0 || k > 0) ? 1u : 0u);
                        }
                    }
                }
                tc::commit(&K->empty[sg]);
            }
        }
    } else {
        // warps 2-5: the built operand and the bias sum
        const int h = warp - 2;
        float* xs = (float*)(smem + 2 * Cfg::STAGE) + h * 9 * WG_WIN;  // WG_FIRST
        constexpr int NR = MODE == WG_FIRST ? (9 * WG_WIN + 31) / 32 : 1;
        float r[NR];  // the next block's global data, in flight
        float bacc = 0.f;
        int64_t t = blockIdx.x;
        if (t < nt) wg_fetch<MODE>(d, t, h, lane, gvec, xin, s, r);
        for (int64_t kb = 0; t < nt && !*abort; t += gridDim.x, kb++) {
            const int sg = (int)(kb & 1);
            uint8_t* st = smem + sg * Cfg::STAGE;
            {
                if (!__all_sync(0xffffffffu,
                                kb < 2 || wait_live(&K->empty[sg],
                                                    (uint32_t)(((kb >> 1) - 1) & 1), abort))) {
                    if (lane == 0) fail();
                    break;
                }
                float cur[NR];
#pragma unroll
                for (int k = 0; k < NR; k++) cur[k] = r[k];
                if (t + gridDim.x < nt) wg_fetch<MODE>(d, t + gridDim.x, h, lane, gvec, xin, s, r);
                const int k = 32 * h + lane;
                if (MODE == WG_LAST) {
                    bacc += cur[0];
                    wg_split_store(st + Cfg::OFF_X, 0, 1, k, cur[0]);
                } else {
                    __syncwarp();  // the previous block's reads of the window are done
#pragma unroll
                    for (int e = 0; e < NR; e++)
                        if (lane + 32 * e < 9 * WG_WIN) xs[lane + 32 * e] = cur[e];
                    __syncwarp();
#pragma unroll
                    for (int q = 0; q < 9; q++)
#pragma unroll
                        for (int dx = 0; dx < 3; dx++)
                            wg_split_store(st + Cfg::OFF_X, 3 * q + dx, 32 + 3 * q + dx, k,
                                           xs[q * WG_WIN + lane + dx]);
                }
                tc::fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&K->bfull[sg]);
            }
            if (MODE != WG_LAST) {
                if (!__all_sync(0xffffffffu,
                                wait_live(&K->tfull[sg], (uint32_t)((kb >> 1) & 1), abort))) {
                    if (lane == 0) fail();
                    break;
                }
                // channel o = lane of x = 32 h .. 32 h + 31, in the gradient
                // copy staged from x0 - 1 (row x + 1)
                const uint8_t* gp = st + Cfg::OFF_G +
                                    (lane >> 3) * WG_PLANE + (lane & 7) * 2;
#pragma unroll 8
                for (int x = 32 * h; x < 32 * h + 32; x++)
                    bacc += __bfloat162float(*(const __nv_bfloat16*)(gp + (x + 1) * 16));
                __syncwarp();
                if (lane == 0) mbar_arrive(&K->empty[sg]);
            }
        }
        K->bsum[h][lane] = bacc;
    }
    // drain: every MMA issued has completed before TMEM is read or released
    __syncthreads();
    if (warp == 1 && lane == 0) tc::commit(&K->drain);
    if (!tc::mbar_wait(&K->drain, 0, WAIT_LIMIT)) tc::mbar_wait(&K->drain, 0, WAIT_LIMIT);
    tc::fence_after();
    const bool ok = *abort == 0;
    float* prow = partial + (int64_t)blockIdx.x * 28 * C;
    auto bias_of = [&](int o) {
        return ((K->bsum[0][o] + K->bsum[1][o]) + K->bsum[2][o]) + K->bsum[3][o];
    };
    if (MODE == WG_FIRST) {
        // rows 32 + tap (lo) of warp 1 meet rows tap (hi) of warp 0
        float* lo = (float*)smem;  // the stages are idle now
        uint32_t acc[32];
        if (ok && warp == 1) {
            tc::ld32(tmem, 32, 0, acc);
            for (int o = 0; o < C; o++) lo[lane * C + o] = __uint_as_float(acc[o]);
        }
        __syncthreads();
        if (ok && warp == 0) {
            tc::ld32(tmem, 0, 0, acc);
            if (lane < 27)
                for (int o = 0; o < C; o++)
                    prow[lane * C + o] = __uint_as_float(acc[o]) + lo[lane * C + o];
        }
        if (ok && warp == 2) prow[27 * C + lane] = bias_of(lane);
    } else if (ok && warp < 4) {
        // TMEM lane 32 w + i of block (gi, dx): strip g0 + w
        for (int gi = 0; gi < 3; gi++) {
            if (gi == 2 && warp < 3) continue;  // strips 5-7 again
            const int q = (gi == 0 ? 0 : (gi == 1 ? 4 : 5)) + warp;
            for (int dx = 0; dx < 3; dx++) {
                uint32_t acc[32];
                tc::ld32(tmem, (uint32_t)(warp * 32), (uint32_t)((gi * 3 + dx) * 32), acc);
                prow[(3 * q + dx) * C + lane] = __uint_as_float(acc[0]) + __uint_as_float(acc[1]);
            }
        }
        if (tid == 0) {
            float sacc = 0.f;
            for (int k = 0; k < 4 * C; k++) sacc += K->bsum[k >> 5][k & 31];
            prow[27 * C] = sacc;
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, Cfg::NCOL);
}

// ---- 32 -> 32 weight gradient walking along y --------------------------------
// dW of a 32 -> 32 layer: the tap's x shift moves onto the gradient (per row of
// the volume, sum_x g[x] a[x + dx - 1] = sum_x' g[x' + 1 - dx] a[x'], both zero
// outside the row), so that with K = x' the input strips are B unshifted (rows
// (strip, i)) and A (M = 128) is the gradient strip in three copies, copy c
// staged from x0 + 1 - c (rows (c, o); copy 3 is zeros): D[(dx, o)][(strip, i)].
// The staging is shared between neighbouring rows, as in conv32_walk_kernel: a CTA takes runs of L rows y of
// one (patch, z, x tile) column; the input strips come as row-sets (the strips
// of one input row in planes z - 1, z, z + 1) through a ring of GW_R slots, each
// row-set loaded once for the three K blocks (output rows) that read it.  Per
// K step three MMAs of N = 96, one per row-set (its three strips; the ring's
// slots are not contiguous), into TMEM columns 96 dy + 32 dz + i.  The
// gradient strip is loaded once per K block (from x0 - 1) and the builder
// warps derive the copies staged from x0 + 1 and x0 (rows shifted by 2 and 1)
// in shared memory; copy 3 stays zero.  About 5.5 strips are staged per K
// block instead of 12.  Roles as in wgrad_tc_kernel; every wait is bounded.
constexpr int GW_R = 5;
constexpr int GW_G = 4 * WG_STRIP;  // one gradient stage: copies 0..3
constexpr int GW_THREADS = 192;

struct GwCtl {
    uint64_t rfull[GW_R], rempty[GW_R], gfull[2], gbuilt[2], gempty[2], drain;
    uint32_t tslot;
    int abort;
    float bsum[4][C];
};

__global__ void __launch_bounds__(GW_THREADS, 1) wgrad_walk_kernel(
    Dims d, WalkPlan wp, const __grid_constant__ CUtensorMap amap,
    const __grid_constant__ CUtensorMap amap_hi, const __grid_constant__ CUtensorMap gmap,
    const __grid_constant__ CUtensorMap gmap_hi, float* __restrict__ partial, int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* ring = smem;
    uint8_t* gst = smem + GW_R * W_SET;
    GwCtl* K = (GwCtl*)(gst + 2 * GW_G);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int k = tid; k < WG_STRIP / 16; k += GW_THREADS) {  // copy 3 of both stages: zeros
        ((uint4*)(gst + 3 * WG_STRIP))[k] = make_uint4(0, 0, 0, 0);
        ((uint4*)(gst + GW_G + 3 * WG_STRIP))[k] = make_uint4(0, 0, 0, 0);
    }
    tc::fence_async_smem();
    if (tid == 0) {
        for (int s = 0; s < GW_R; s++) {
            tc::mbar_init(&K->rfull[s], 1);
            tc::mbar_init(&K->rempty[s], 1);
        }
        for (int s = 0; s < 2; s++) {
            tc::mbar_init(&K->gfull[s], 1);
            tc::mbar_init(&K->gbuilt[s], 4);
            tc::mbar_init(&K->gempty[s], 1);
        }
        tc::mbar_init(&K->drain, 1);
        K->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::tmem_alloc(&K->tslot, 512);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = K->tslot;
    volatile int* abort = &K->abort;
    auto fail = [&]() {
        if (!*abort) atomicOr(status, NR_FLAG_TIMEOUT);
        *abort = 1;
        __threadfence_block();
    };
    auto strip_ok = [&](int zz, int yy) { return zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny; };
    if (warp == 0) {
        if (lane == 0) {
            // producer: per item row-sets 0 and 1, then per K block i row-set
            // i + 2 and the gradient strip
            int64_t G = 0, kb = 0, rissued = 0, kissued = 0;
            bool stop = false;
            auto load_set = [&](int b, int z, int x0, int Y) {
                const int s = (int)(G % GW_R);
                if (G >= GW_R &&
                    !wait_live(&K->rempty[s], (uint32_t)((G / GW_R - 1) & 1), abort))
                    return false;
                mbar_arrive_tx(&K->rfull[s], 3 * STRIP_TX);
                for (int dz = 0; dz < 3; dz++)
                    load_strip(ring + s * W_SET + dz * TSTRIP, PLANE, &amap, &amap_hi, x0,
                               strip_ok(z + dz - 1, Y) ? (b * d.nz + z + dz - 1) * d.ny + Y : -1,
                               &K->rfull[s]);
                rissued = ++G;
                return true;
            };
            for (int64_t it = blockIdx.x; it < wp.nitems && !stop && !*abort; it += gridDim.x) {
                int b, z, x0, y0, ly;
                item_pos(d, wp, it, b, z, x0, y0, ly);
                if (!load_set(b, z, x0, y0 - 1) || !load_set(b, z, x0, y0)) {
                    fail();
                    break;
                }
                for (int i = 0; i < ly; i++, kb++) {
                    if (!load_set(b, z, x0, y0 + i + 1)) {
                        fail();
                        stop = true;
                        break;
                    }
                    const int gs = (int)(kb & 1);
                    if (kb >= 2 && !wait_live(&K->gempty[gs], (uint32_t)(((kb >> 1) - 1) & 1), abort)) {
                        fail();
                        stop = true;
                        break;
                    }
                    mbar_arrive_tx(&K->gfull[gs], STRIP_TX);
                    load_strip(gst + gs * GW_G + 2 * WG_STRIP, PLANE, &gmap, &gmap_hi, x0,
                               (b * d.nz + z) * d.ny + y0 + i, &K->gfull[gs]);
                    kissued = kb + 1;
                }
            }
            // no copy may be in flight when the block exits
            for (int64_t k = rissued > GW_R ? rissued - GW_R : 0; k < rissued; k++) {
                uint64_t* bar = &K->rfull[k % GW_R];
                if (!tc::mbar_wait(bar, (uint32_t)((k / GW_R) & 1), WAIT_LIMIT))
                    tc::mbar_wait(bar, (uint32_t)((k / GW_R) & 1), WAIT_LIMIT);
            }
            for (int64_t k = kissued > 2 ? kissued - 2 : 0; k < kissued; k++) {
                uint64_t* bar = &K->gfull[k & 1];
                if (!tc::mbar_wait(bar, (uint32_t)((k >> 1) & 1), WAIT_LIMIT))
                    tc::mbar_wait(bar, (uint32_t)((k >> 1) & 1), WAIT_LIMIT);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer.  Test hook: the workspace's second status word k + 1
            // > 0 makes the wait for this CTA's K block k report giving up
            // once it has in fact succeeded.
            const int force_at = status[1] - 1;
            constexpr uint32_t idesc = tc::idesc_bf16(TM, 96) | (1u << 15) | (1u << 16);
            const uint64_t ad0 = tc::sdesc(tc::smem_u32(gst), 128, WG_PLANE);
            const uint64_t bd0 = tc::sdesc(tc::smem_u32(ring), 128, WG_PLANE);
            int64_t G = 0, kb = 0;
            bool stop = false;
            for (int64_t it = blockIdx.x; it < wp.nitems && !stop && !*abort; it += gridDim.x) {
                int b, z, x0, y0, ly;
                item_pos(d, wp, it, b, z, x0, y0, ly);
                for (int i = 0; i < ly; i++, kb++) {
                    const int gs = (int)(kb & 1);
                    bool got = wait_live(&K->gbuilt[gs], (uint32_t)((kb >> 1) & 1), abort);
                    int slot[3];
                    for (int dy = 0; dy < 3 && got; dy++) {
                        const int64_t g2 = G + i + dy;
                        slot[dy] = (int)(g2 % GW_R);
                        if (i == 0 || dy == 2)
                            got = wait_live(&K->rfull[slot[dy]], (uint32_t)((g2 / GW_R) & 1), abort);
                    }
                    if (kb == force_at) got = false;
                    if (!got) {
                        fail();
                        stop = true;
                        break;
                    }
                    tc::fence_after();
                    const uint64_t adg = ad0 + (uint64_t)((gs * GW_G) >> 4);
#pragma unroll
                    for (int ks = 0; ks < TM / 16; ks++)
#pragma unroll
                        for (int dy = 0; dy < 3; dy++)
                            tc::mma_bf16(tmem + (uint32_t)(dy * 96),
                                         adg + (uint64_t)((ks * 256) >> 4),
                                         bd0 + (uint64_t)((slot[dy] * W_SET + 16 + ks * 256) >> 4),
                                         idesc, (kb > 0 || ks > 0) ? 1u : 0u);
                    tc::commit(&K->gempty[gs]);
                    // row-set i is not read after this K block; the last one of
                    // the item also frees row-sets ly and ly + 1
                    tc::commit(&K->rempty[slot[0]]);
                    if (i == ly - 1) {
                        tc::commit(&K->rempty[slot[1]]);
                        tc::commit(&K->rempty[slot[2]]);
                    }
                }
                G += ly + 2;
            }
        }
    } else {
        // warps 2-5: the shifted gradient copies and the bias sum
        const int h = warp - 2;
        float bacc = 0.f;
        int64_t kb = 0;
        bool stop = false;
        for (int64_t it = blockIdx.x; it < wp.nitems && !stop && !*abort; it += gridDim.x) {
            int b, z, x0, y0, ly;
            item_pos(d, wp, it, b, z, x0, y0, ly);
            for (int i = 0; i < ly; i++, kb++) {
                const int gs = (int)(kb & 1);
                if (!__all_sync(0xffffffffu,
                                wait_live(&K->gfull[gs], (uint32_t)((kb >> 1) & 1), abort))) {
                    if (lane == 0) fail();
                    stop = true;
                    break;
                }
                uint8_t* st = gst + gs * GW_G;
                // copy c (c = 0, 1) row r = copy 2 row r + 2 - c, r < 128: 8 planes
                // x 128 rows of 16 bytes over the 128 builder threads
                const int t = h * 32 + lane;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const int u = k * 128 + t;  // 0 .. 1023
                    const int c = u >> 9, p = (u >> 7) & 3, r = u & 127;
                    const uint4 v = *(const uint4*)(st + 2 * WG_STRIP + p * WG_PLANE + (r + 2 - c) * 16);
                    *(uint4*)(st + c * WG_STRIP + p * WG_PLANE + r * 16) = v;
                }
                // channel o = lane of x = 32 h .. 32 h + 31 (copy 2, row x + 1)
                const uint8_t* gp = st + 2 * WG_STRIP + (lane >> 3) * WG_PLANE + (lane & 7) * 2;
#pragma unroll 8
                for (int x = 32 * h; x < 32 * h + 32; x++)
                    bacc += __bfloat162float(*(const __nv_bfloat16*)(gp + (x + 1) * 16));
                tc::fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&K->gbuilt[gs]);
            }
        }
        K->bsum[h][lane] = bacc;
    }
    // drain: every MMA issued has completed before TMEM is read or released
    __syncthreads();
    if (warp == 1 && lane == 0) tc::commit(&K->drain);
    if (!tc::mbar_wait(&K->drain, 0, WAIT_LIMIT)) tc::mbar_wait(&K->drain, 0, WAIT_LIMIT);
    tc::fence_after();
    const bool ok = *abort == 0;
    float* prow = partial + (int64_t)blockIdx.x * 28 * C * C;
    // TMEM lane 32 dx + o, column 96 dy + 32 dz + i: dW[9 dz + 3 dy + dx][o][i]
    if (ok && warp < 3) {
        for (int dy = 0; dy < 3; dy++)
            for (int dz = 0; dz < 3; dz++) {
                uint32_t acc[32];
                tc::ld32(tmem, (uint32_t)(warp * 32), (uint32_t)(dy * 96 + dz * 32), acc);
                float4* dst = (float4*)(prow + ((dz * 9 + dy * 3 + warp) * C + lane) * C);
#pragma unroll
                for (int j = 0; j < 8; j++)
                    dst[j] = make_float4(__uint_as_float(acc[4 * j]), __uint_as_float(acc[4 * j + 1]),
                                         __uint_as_float(acc[4 * j + 2]),
                                         __uint_as_float(acc[4 * j + 3]));
            }
    }
    if (ok && warp == 3)
        prow[(27 * C + lane) * C] =
            ((K->bsum[0][lane] + K->bsum[1][lane]) + K->bsum[2][lane]) + K->bsum[3][lane];
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// grad[tap][o][i] (and grad_b[o] from tap 27, i = 0) = the sum of the CTAs'
// partials (partial[cta][e], e = tap nout + o ni + i).  A block of 8 warps
// takes 32 consecutive e: warp w adds, in CTA order, the CTAs of its eighth of
// the range for the lane's e (coalesced rows), and warp 0 adds the eight
// subtotals in warp order -- a fixed order for a given CTA count.
__global__ void __launch_bounds__(256) wgrad_reduce_kernel(const float* __restrict__ partial,
                                                           int64_t nchunk, int nout, int ni,
                                                           float* __restrict__ gw,
                                                           float* __restrict__ gb) {
    __shared__ double sub[8][32];
    const int64_t n = 28LL * nout;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t e = (int64_t)blockIdx.x * 32 + lane;
    const int64_t c0 = nchunk * w / 8, c1 = nchunk * (w + 1) / 8;
    double s = 0.0;
    if (e < n) {
        int64_t c = c0;
        for (; c + 4 <= c1; c += 4) {
            const float a0 = partial[c * n + e], a1 = partial[(c + 1) * n + e];
            const float a2 = partial[(c + 2) * n + e], a3 = partial[(c + 3) * n + e];
            s += a0;
            s += a1;
            s += a2;
            s += a3;
        }
        for (; c < c1; c++) s += partial[c * n + e];
    }
    sub[w][lane] = s;
    __syncthreads();
    if (w == 0 && e < n) {
        double t = 0.0;
        for (int k = 0; k < 8; k++) t += sub[k][lane];
        const int tap = (int)(e / nout), oi = (int)(e % nout);
        if (tap < 27) gw[e] = (float)t;
        else if (oi % ni == 0) gb[oi / ni] = (float)t;
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
// mode 4: forward of the 1-output layer in row passes: per dx one 16 x 32
//         block, row n = (dz, dy) = 3 dz + dy (n < 9), k = i, from
//         W[9 dz + 3 dy + dx][0][i].
__global__ void pack_kernel(const float* __restrict__ w, int mode, int NI, int NO, int NOUT,
                            __nv_bfloat16* __restrict__ out) {
    const int per_tap = NOUT * C;
    const int total = (mode == 2 || mode == 3) ? C * C : (mode == 4 ? 3 * 16 * C : 27 * per_tap);
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
        } else if (mode == 3) {
            const int n = e / C, k = e % C;
            if (k < 27 && n < NI) v = w[((int64_t)(26 - k) * NO + 0) * NI + n];
            dst = bpk_index(n, k);
        } else {
            const int dx = e / (16 * C), r = e % (16 * C), n = r / C, k = r % C;
            if (n < 9) v = w[((int64_t)((n / 3) * 9 + (n % 3) * 3 + dx) * NO + 0) * NI + k];
            dst = dx * 16 * C + bpk_index(n, k);
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

// One warp: lane l adds partials l, l + 32, ...; then a fixed shuffle tree.
__global__ void loss_final_kernel(const double* __restrict__ partial, int n, int64_t V,
                                  double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    double t = 0.0;
    for (int k = lane; k < n; k += 32) t += partial[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) out[0] = t / (double)V;
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
    L.nchunk = ntiles(d) < WG_MAXCTA ? ntiles(d) : WG_MAXCTA;  // CTAs of a weight gradient
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

// The TMA maps of an activation tensor (act_off's layout) seen as (2 nx
// 8-byte units, 4 K chunks, R rows): one K chunk of a row is one contiguous
// run; `lo` boxes are 128 units (strip rows 0-63), `hi` boxes 132 units (rows
// 64-129).  Zeros outside the tensor.
struct ActMaps {
    CUtensorMap lo, hi;
};
static bool act_maps(const Dims& d, const __nv_bfloat16* in, ActMaps* m) {
    auto enc = tensor_map_encode_fn();
    if (!enc || ((uintptr_t)in & 15) != 0) return false;
    const cuuint64_t rows = (cuuint64_t)d.ny * d.nz * d.nb;
    const cuuint64_t dims[3] = {(cuuint64_t)d.nx * 2, (cuuint64_t)KCH, rows};
    const cuuint64_t strides[2] = {(cuuint64_t)d.nx * 16, (cuuint64_t)d.nx * C * 2};
    const cuuint32_t estr[3] = {1, 1, 1};
    const cuuint32_t box_lo[3] = {128, 1, 1}, box_hi[3] = {132, 1, 1};
    auto one = [&](CUtensorMap* map, const cuuint32_t* box) {
        return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, (void*)in, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    };
    return one(&m->lo, box_lo) && one(&m->hi, box_hi);
}

template <int NOUT, int EPI>
static nr_status launch_conv32(const Dims& d, const __nv_bfloat16* in, const __nv_bfloat16* wpk,
                               const float* bias, void* out, const __nv_bfloat16* mask,
                               int* status, cudaStream_t s) {
    ActMaps map;
    if (!act_maps(d, in, &map)) return NR_ERR_CUDA;  // the input cannot be described for TMA
    // runs of L rows: about eight items per SM, L in [4, 32]
    const int nsm = sm_count();
    const int64_t ncols = (int64_t)d.nb * d.nz * xtiles(d);
    int64_t L = ((int64_t)d.ny * ncols + 8LL * nsm - 1) / (8LL * nsm);
    L = L < 4 ? 4 : (L > 32 ? 32 : L);
    if (L > d.ny) L = d.ny;
    WalkPlan wp;
    wp.L = (int)L;
    wp.nchunk = (int)((d.ny + L - 1) / L);
    const int grid_max = nsm;
    // The dx-stacked kernel costs about 0.6 of the other per row of tiles
    // (whole network on 512 x 60 planes: 1.46 against 2.36 ms at one tile per
    // row, nx = 126 / 128; 2.73 against 4.60 ms at two, nx = 252 / 256) but
    // needs ceil(nx / 126) tiles per row: it is used when that is cheaper
    // (not for nx = 128, where two of its tiles cost 2.73 ms against 2.36).
    const int t126 = (d.nx + W3_TW - 1) / W3_TW, t128 = (d.nx + TM - 1) / TM;
    if (60 * t126 < 100 * t128) {
        wp.tw = W3_TW;
        wp.nitems = (int64_t)d.nb * d.nz * t126 * wp.nchunk;
        const size_t smem = (size_t)W_R * W_SET + 27 * NOUT * C * 2 + sizeof(W3Ctl);
        if (cudaFuncSetAttribute(conv32_w3_kernel<NOUT, EPI>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return NR_ERR_CUDA;
        const int grid = (int)(wp.nitems < (int64_t)grid_max ? wp.nitems : (int64_t)grid_max);
        conv32_w3_kernel<NOUT, EPI><<<grid, W3_THREADS, smem, s>>>(d, wp, map.lo, map.hi, wpk,
                                                                   bias, out, mask, status);
        return launch_status();
    }
    wp.tw = TM;
    wp.nitems = (int64_t)d.nb * d.nz * t128 * wp.nchunk;
    const size_t smem = (size_t)W_R * W_SET + 27 * NOUT * C * 2 + sizeof(WalkCtl);
    if (cudaFuncSetAttribute(conv32_walk_kernel<NOUT, EPI>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return NR_ERR_CUDA;
    const int grid = (int)(wp.nitems < (int64_t)grid_max ? wp.nitems : (int64_t)grid_max);
    conv32_walk_kernel<NOUT, EPI><<<grid, W_THREADS, smem, s>>>(d, wp, map.lo, map.hi, wpk, bias,
                                                                out, mask, status);
    return launch_status();
}

template <int EPI>
static nr_status launch_conv1(const Dims& d, const float* in, float scale,
                              const __nv_bfloat16* wpk, const float* bias, void* out,
                              const __nv_bfloat16* mask, int* status, cudaStream_t s) {
    // four CTAs per SM (nine, as many as fit, measured 2.7x slower on the
    // clinical volume), each walking runs of L rows: about eight runs per CTA
    const int nsm = sm_count();
    const int64_t ncols = (int64_t)d.nb * d.nz * xtiles(d);
    int64_t L = ((int64_t)d.ny * ncols + 32LL * nsm - 1) / (32LL * nsm);
    L = L < 1 ? 1 : (L > 32 ? 32 : L);
    if (L > d.ny) L = d.ny;
    WalkPlan wp;
    wp.L = (int)L;
    wp.nchunk = (int)((d.ny + L - 1) / L);
    wp.tw = TM;
    wp.nitems = ncols * wp.nchunk;
    const int grid = (int)(wp.nitems < (int64_t)nsm * 4 ? wp.nitems : (int64_t)nsm * 4);
    conv1_kernel<EPI><<<grid, 128, 0, s>>>(d, wp, in, scale, wpk, bias, out, mask, status);
    return launch_status();
}

// The 32 -> 1 layer (two passes); q: 9 V floats of scratch.
static nr_status launch_last(const Dims& d, const __nv_bfloat16* in, const __nv_bfloat16* wpk,
                             const float* bias, float* q, float* f, int* status, cudaStream_t s) {
    ActMaps map;
    if (!act_maps(d, in, &map)) return NR_ERR_CUDA;
    const size_t smem = (size_t)LR_STAGE * TSTRIP + 3 * 16 * C * 2 + sizeof(LastCtl);
    if (cudaFuncSetAttribute(last_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return NR_ERR_CUDA;
    const int64_t nt = ntiles(d);
    const int grid = (int)(nt < (int64_t)sm_count() * 4 ? nt : (int64_t)sm_count() * 4);
    last_rows_kernel<<<grid, LR_THREADS, smem, s>>>(d, map.lo, map.hi, wpk, q, status);
    // q planes start at multiples of V floats: with nx % 4 == 0 every row is 16-byte
    // aligned (the workspace is 256-byte aligned)
    if (d.nx % 4 == 0) {
        const dim3 g2((unsigned)((int64_t)d.nb * d.nz * d.ny), (unsigned)((d.nx / 4 + 255) / 256));
        last_sum_kernel<4><<<g2, 256, 0, s>>>(d, q, bias, f);
    } else {
        const dim3 g2((unsigned)((int64_t)d.nb * d.nz * d.ny), (unsigned)((d.nx + 255) / 256));
        last_sum_kernel<1><<<g2, 256, 0, s>>>(d, q, bias, f);
    }
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
    pack(params + wo[5], 4, C, 1, 16, pkf(5), st);
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
    // q of the last layer: a buffer idle by now (the gradient buffer when the
    // activations are kept for training, else layer 4's ping-pong buffer)
    float* q = (float*)(ws + (keep ? L.dpre[0] : L.act[1]));
    return launch_last(d, act(4), pkf(5), params + bo[5], q, (float*)(ws + L.f), status, st);
}

__global__ void target_kernel(const float* __restrict__ x, const float* __restrict__ t, float s,
                              int64_t V, float* __restrict__ r) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V;
         v += (int64_t)gridDim.x * blockDim.x)
        r[v] = s * (t[v] - x[v]);
}

template <int MODE>
static nr_status launch_wgrad(const Dims& d, const ActMaps& am, const ActMaps& gm,
                              const float* gvec, const float* xin, float s, float* part,
                              int* status, int64_t nch, cudaStream_t st) {
    if (cudaFuncSetAttribute(wgrad_tc_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             WgCfg<MODE>::SMEM) != cudaSuccess)
        return NR_ERR_CUDA;
    wgrad_tc_kernel<MODE><<<(unsigned)nch, WG_THREADS, WgCfg<MODE>::SMEM, st>>>(
        d, am.lo, am.hi, gm.lo, gm.hi, gvec, xin, s, part, status);
    return launch_status();
}

// Weight and bias gradients of layer l (0-based) into grad: the tensor-core
// GEMM (one partial per CTA), then the fixed-order reduction.  Layer 0 reads
// the FP32 input volume (times s), layer 5 the FP32 gradient of the output.
static nr_status wgrad(const Dims& d, int l, const void* g, const void* in, float s, char* ws,
                       const WSL& L, float* grad, int* status, cudaStream_t st) {
    int64_t wo[6], bo[6], P;
    param_offsets(wo, bo, &P);
    float* part = (float*)(ws + L.part);
    const int64_t nt = ntiles(d);
    int64_t nch = nt < (int64_t)sm_count() ? nt : (int64_t)sm_count();
    if (nch > L.nchunk) nch = L.nchunk;
    ActMaps am{}, gm{};  // a map a mode does not read stays zero
    if (l > 0 && !act_maps(d, (const __nv_bfloat16*)in, &am)) return NR_ERR_CUDA;
    if (l < 5 && !act_maps(d, (const __nv_bfloat16*)g, &gm)) return NR_ERR_CUDA;
    nr_status e;
    int nout = C, ni = C;
    if (l == 0) {
        e = launch_wgrad<WG_FIRST>(d, am, gm, nullptr, (const float*)in, s, part, status, nch, st);
        ni = 1;
    } else if (l == 5) {
        e = launch_wgrad<WG_LAST>(d, am, gm, (const float*)g, nullptr, 1.f, part, status, nch, st);
    } else {
        // runs of L rows along y: about eight per CTA
        int64_t L = ((int64_t)d.ny * d.nb * d.nz * xtiles(d) + 8 * nch - 1) / (8 * nch);
        L = L < 4 ? 4 : (L > 32 ? 32 : L);
        if (L > d.ny) L = d.ny;
        WalkPlan wp;
        wp.L = (int)L;
        wp.nchunk = (int)((d.ny + L - 1) / L);
        wp.tw = TM;
        wp.nitems = (int64_t)d.nb * d.nz * xtiles(d) * wp.nchunk;
        if (wp.nitems < nch) nch = wp.nitems;
        const size_t smem = (size_t)GW_R * W_SET + 2 * GW_G + sizeof(GwCtl);
        if (cudaFuncSetAttribute(wgrad_walk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return NR_ERR_CUDA;
        wgrad_walk_kernel<<<(unsigned)nch, GW_THREADS, smem, st>>>(d, wp, am.lo, am.hi, gm.lo,
                                                                   gm.hi, part, status);
        e = launch_status();
        nout = C * C;
    }
    if (e != NR_OK) return e;
    wgrad_reduce_kernel<<<(28 * nout + 31) / 32, 256, 0, st>>>(part, nch, nout, ni, grad + wo[l],
                                                               grad + bo[l]);
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
