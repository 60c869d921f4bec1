// update.cuh -- the fused OSTR update of one tile (device code shared by the
// single-reconstruction kernel in prior.cu and the batched kernel in batch.cu).
//
// Per voxel and in one pass:
//     capL = M * SBP(h over the subset views)          (Tomo_OSTR_gold.cpp:759-771)
//     RDD, RD = 26-neighbour penalty sums of x         (:775, Tomo_OSTR.cu:118-325)
//     x' = max(0, x - (capL + beta RD) / (d + 2 beta RDD))   (update_est :265-295)
#pragma once

#include <cmath>

#include "common.cuh"
#include "tma.cuh"

namespace nr {

constexpr int UPD_VIEWS_SMEM = 32;
constexpr int UTX = 32, UTY = 8, UZC = 16;      // tile: 32 x 8 columns, 16 planes per block
constexpr int USW = UTX + 2, USH = UTY + 2;     // plane tile with a 1-voxel halo
constexpr int UPLANE = USW * USH;

// The five distinct neighbour weights 1/sqrt(dx^2+dy^2+(dz zr)^2) of the
// 26-neighbourhood (in-plane face, in-plane diagonal, z face, z edge, z
// corner), the same times delta (Huber), 1/delta and 1, each duplicated into
// both halves of a packed FP32 pair: the penalty works on neighbour pairs
// (nb_pair), and a pair operand read whole from the constant bank costs no
// instruction to assemble.
enum { W_FACE, W_DIAG, W_ZFACE, W_ZEDGE, W_ZCORNER, W_CLASSES };
struct alignas(8) PriorW5 {
    float2 w[W_CLASSES];   // weight of each class
    float2 wd[W_CLASSES];  // weight x delta
    float2 inv_delta;      // 1 / delta (hyperbola)
    float2 one;
};

__host__ inline PriorW5 make_w5(float zxy, float delta) {
    auto w = [&](int dx, int dy, int dz) {
        const float dist = std::sqrt((float)(dx * dx + dy * dy) + (float)(dz * dz) * zxy * zxy);
        return (float)(1.0 / (double)dist);
    };
    const float cls[W_CLASSES] = {w(1, 0, 0), w(1, 1, 0), w(0, 0, 1), w(1, 0, 1), w(1, 1, 1)};
    PriorW5 p;
    for (int k = 0; k < W_CLASSES; k++) {
        p.w[k] = make_float2(cls[k], cls[k]);
        p.wd[k] = make_float2(cls[k] * delta, cls[k] * delta);
    }
    const float idl = 1.f / delta;
    p.inv_delta = make_float2(idl, idl);
    p.one = make_float2(1.f, 1.f);
    return p;
}

// Approximate reciprocal / reciprocal square root (the MUFU unit, <= 1 ulp
// relative error; arguments here are >= 1 or >= delta, never denormal).
__device__ __forceinline__ float rcp_approx(float v) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float v) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}

// Packed FP32 pairs (add / sub / mul / fma on .f32x2): two neighbour terms per
// instruction, each lane rounded as the scalar operation would be.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(f32x2 r, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
// A duplicated pair stored as float2, read as one 64-bit value.
__device__ __forceinline__ f32x2 ld2(const float2& v) {
    return *reinterpret_cast<const f32x2*>(&v);
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Weight class of neighbour K = ((dz+1)*3 + (dy+1))*3 + (dx+1).
template <int K>
__device__ __forceinline__ constexpr int nb_class() {
    constexpr int dz = K / 9 - 1, dy = (K / 3) % 3 - 1, dx = K % 3 - 1;
    constexpr int nxy = (dx != 0) + (dy != 0);
    return dz == 0 ? (nxy == 1 ? W_FACE : W_DIAG)
                   : (nxy == 0 ? W_ZFACE : (nxy == 1 ? W_ZEDGE : W_ZCORNER));
}

// The penalty terms of a packed pair of differences t2 of one weight class:
// each lane adds w omega(t) to sdd and w omega(t) t to sd.  EDGE: a
// difference with an out-of-volume cell (NaN) counts as t = 0.
template <int POT, bool EDGE, int CLS>
__device__ __forceinline__ void nb_terms(f32x2 t2, const PriorW5& W, float delta, float inv_delta,
                                         f32x2& sdd, f32x2& sd) {
    float ta, tb;
    upk2(t2, ta, tb);
    if (EDGE) {
        ta = (ta == ta) ? ta : 0.f;
        tb = (tb == tb) ? tb : 0.f;
        t2 = pk2(ta, tb);
    }
    const f32x2 w2 = ld2(W.w[CLS]);
    f32x2 wo2;
    if (POT == NR_POT_Q2) {
        wo2 = w2;
    } else if (POT == NR_POT_LANGE) {
        wo2 = mul2(w2, pk2(rcp_approx(__fmaf_rn(fabsf(ta), inv_delta, 1.f)),
                           rcp_approx(__fmaf_rn(fabsf(tb), inv_delta, 1.f))));
    } else if (POT == NR_POT_HYPERBOLA) {
        const f32x2 u2 = mul2(t2, ld2(W.inv_delta));
        float qa, qb;
        upk2(fma2(u2, u2, ld2(W.one)), qa, qb);
        wo2 = mul2(w2, pk2(rsqrt_approx(qa), rsqrt_approx(qb)));
    } else {
        wo2 = mul2(ld2(W.wd[CLS]), pk2(rcp_approx(fmaxf(fabsf(ta), delta)),
                                       rcp_approx(fmaxf(fabsf(tb), delta))));
    }
    sdd = add2(sdd, wo2);
    sd = fma2(wo2, t2, sd);
}

// Neighbours KA and KB (same weight class) of the centre at offset `base` in
// the shared-memory planes, in one packed step: lane 0 accumulates KA's
// terms, lane 1 KB's.  Against one neighbour per step this saves the
// difference, the weight product and both accumulations of every second
// neighbour (5 instead of 7 instructions per Huber term, 5.5 instead of 8 per
// hyperbola term; measured 5 % / 8 % off the update).
template <int POT, bool EDGE, int KA, int KB, int RW = USW>
__device__ __forceinline__ void nb_pair(const float* __restrict__ pb, const float* __restrict__ pc,
                                        const float* __restrict__ pa, int base, f32x2 xc2,
                                        const PriorW5& W, float delta, float inv_delta,
                                        f32x2& sdd, f32x2& sd) {
    constexpr int dza = KA / 9 - 1, dya = (KA / 3) % 3 - 1, dxa = KA % 3 - 1;
    constexpr int dzb = KB / 9 - 1, dyb = (KB / 3) % 3 - 1, dxb = KB % 3 - 1;
    static_assert(nb_class<KA>() == nb_class<KB>(), "one weight class");
    const float* pla = dza < 0 ? pb : (dza == 0 ? pc : pa);
    const float* plb = dzb < 0 ? pb : (dzb == 0 ? pc : pa);
    const f32x2 t2 = sub2(xc2, pk2(pla[base + dya * RW + dxa], plb[base + dyb * RW + dxb]));
    nb_terms<POT, EDGE, nb_class<KA>()>(t2, W, delta, inv_delta, sdd, sd);
}

// The 26 neighbours as 13 equal-weight pairs: (dx = -1, dx = +1) of each
// (dy, dz) row, and the dx = 0 cells paired across dy or dz.  RW: floats per
// row of the staged planes.
template <int POT, bool EDGE, int RW>
__device__ __forceinline__ void prior_pairs_w(const float* __restrict__ pb,
                                              const float* __restrict__ pc,
                                              const float* __restrict__ pa, int base, float xc,
                                              const PriorW5& W, float delta, float inv_delta,
                                              float* rdd, float* rd) {
    const f32x2 xc2 = pk2(xc, xc);
    f32x2 sdd = pk2(0.f, 0.f), sd = pk2(0.f, 0.f);
#define NR_PAIR(a, b) \
    nb_pair<POT, EDGE, a, b, RW>(pb, pc, pa, base, xc2, W, delta, inv_delta, sdd, sd)
    NR_PAIR(0, 2); NR_PAIR(3, 5); NR_PAIR(6, 8);      // dz = -1 rows
    NR_PAIR(9, 11); NR_PAIR(12, 14); NR_PAIR(15, 17); // dz = 0 rows
    NR_PAIR(18, 20); NR_PAIR(21, 23); NR_PAIR(24, 26);  // dz = +1 rows
    NR_PAIR(1, 7); NR_PAIR(19, 25); NR_PAIR(4, 22); NR_PAIR(10, 16);
#undef NR_PAIR
    float a0, a1, b0, b1;
    upk2(sdd, a0, a1);
    upk2(sd, b0, b1);
    *rdd = a0 + a1;
    *rd = b0 + b1;
}

template <int POT, bool EDGE>
__device__ __forceinline__ void prior_pairs(const float* __restrict__ pb,
                                            const float* __restrict__ pc,
                                            const float* __restrict__ pa, int base, float xc,
                                            const PriorW5& W, float delta, float inv_delta,
                                            float* rdd, float* rd) {
    prior_pairs_w<POT, EDGE, USW>(pb, pc, pa, base, xc, W, delta, inv_delta, rdd, rd);
}

// Kinds of fused update (template argument KIND of update_tile).
constexpr int UPD_OSTR = 0;     // OSTR step above
constexpr int UPD_SART = 1;     // OS-SART, backprj_OSSART_gpu_manyviews (Tomo_OSTR.cu:1737-1936)
constexpr int UPD_SART_R = 2;   // OS-SART with the hyperbola prior, backprj_OSSART_R (:1938-2143)

// Shared memory of one update tile: the 3-plane ring and the subset's sources.
struct UpdSmem {
    float tile[3][UPLANE];
    ViewSrc sv[UPD_VIEWS_SMEM];
};

// The back projection of a voxel onto one view's detector is separable: on a
// plane z, the detector column (ilb, fracI) of a voxel depends only on its x
// and the row (jlb, fracJ) only on its y (the ray from the source through
// the voxel centre meets the detector plane at x0 + (x1 - x0) t(z), y0 +
// (y1 - y0) t(z)).  Neither depends on the volume, so they are tabulated once
// per reconstruction, per view (subset order), plane and column / row, with
// the arithmetic of bp.cu's sbp_term in reciprocal-multiply form, as a tap
// pair and its weights:
//   x[(a nz + z) nx + i] = {c, w0, w1, (x0 - x1)^2}
//   y[(a nz + z) ny + j] = {r * BINSx, v0, v1, (y0 - y1)^2 + (z0 - z1)^2}
// The bilinear stencil's columns are ilb, ilb + 1 with weights 1 - fracI,
// fracI; a column off the detector gets weight 0 (the rules of
// Tomo_OSTR.cu:1684-1715), and c is ilb clamped to [0, BINSx - 2] with the
// weights moved to the columns they belong to, so both loads of a pair are
// in bounds and need no test.  Rows likewise (both weights 0 when the plane
// holds the source, :1643).  Interior taps compute exactly what the masked
// stencil did; an edge tap adds w * h + 0 * h' = w * h.  With a detector one
// bin wide (or high) the second load of a pair lands up to BINSx + 1 floats
// past the subset's views: the h sections carry that many zeros (bp_pad).
// Each update reads one entry of each per voxel and view (the x entries of a
// warp are consecutive, its y entry is one broadcast); the tables of a subset
// stay in L2.
struct BpTab {
    const float4* __restrict__ x;
    const float4* __restrict__ y;
};

__device__ __forceinline__ float bp_tt(const nr_geom& g, const ViewSrc& vs, float z1) {
    return z1 != vs.z0 ? __fdividef(-g.detectorR - vs.z0, z1 - vs.z0) : 0.f;
}

// The tables are indexed in 32 bits: true when both hold fewer than 2^31
// entries (the device-resident paths refuse a geometry otherwise).
__host__ inline bool bp_tables_fit(const nr_geom& g) {
    const int64_t n = (int64_t)g.n_angles * g.nz * (g.nx > g.ny ? g.nx : g.ny);
    return n < ((int64_t)1 << 31);
}

// Floats of zero padding after an h section (see the tables above).
__host__ __device__ inline int64_t bp_pad(const nr_geom& g) { return (int64_t)g.nbx + 1; }

// The tap pair (c, c + 1) of two taps at (lb, lb + 1) with weights (w0, w1)
// on a line of n detector bins, weights of off-detector taps already 0.
__device__ __forceinline__ void bp_pair(int lb, float w0, float w1, int n, int& c, float& p0,
                                        float& p1) {
    c = max(0, min(n - 2, lb));
    if (lb == c) {
        p0 = w0;
        p1 = w1;
    } else if (lb == c - 1) {  // lb = -1: only tap lb + 1 = c can be on the detector
        p0 = w1;
        p1 = 0.f;
    } else if (lb == c + 1) {  // lb = n - 1 (n >= 2): only tap lb = c + 1
        p0 = 0.f;
        p1 = w0;
    } else {                   // both taps off the detector (w0 = w1 = 0)
        p0 = 0.f;
        p1 = 0.f;
    }
}

__device__ __forceinline__ float4 bp_entry_x(const nr_geom& g, const ViewSrc& vs, float tt,
                                             int i, float inv_bx) {
    const float x1 = vox_x(g, i);
    const float ddx = vs.x0 - x1;
    const float x2 = vs.x0 + (x1 - vs.x0) * tt;
    const float imb = (x2 - g.x_d0) * inv_bx;
    int ilb = (int)floorf(imb);
    if (imb < (float)ilb + 0.5f) ilb -= 1;
    const float fracI = imb - ((float)ilb + 0.5f);
    const bool i0 = (ilb < g.nbx) && (ilb >= 0);
    const bool i1 = (ilb < g.nbx - 1) && (ilb >= -1);
    int c;
    float p0, p1;
    bp_pair(ilb, i0 ? 1.f - fracI : 0.f, i1 ? fracI : 0.f, g.nbx, c, p0, p1);
    return make_float4(__int_as_float(c), p0, p1, ddx * ddx);
}

__device__ __forceinline__ float4 bp_entry_y(const nr_geom& g, const ViewSrc& vs, float z1,
                                             float tt, int j, float inv_by) {
    const bool valid = z1 != vs.z0;
    const float y1 = vox_y(g, j);
    const float ddy = vs.y0 - y1, ddz = vs.z0 - z1;
    const float y2 = vs.y0 + (y1 - vs.y0) * tt;
    const float jmb = (y2 - g.y_d0) * inv_by;
    int jlb = (int)floorf(jmb);
    if (jmb < (float)jlb + 0.5f) jlb -= 1;
    const float fracJ = jmb - ((float)jlb + 0.5f);
    const bool j0 = valid && (jlb < g.nby) && (jlb >= 0);
    const bool j1 = valid && (jlb < g.nby - 1) && (jlb >= -1);
    int r;
    float p0, p1;
    bp_pair(jlb, j0 ? 1.f - fracJ : 0.f, j1 ? fracJ : 0.f, g.nby, r, p0, p1);
    return make_float4(__int_as_float(r * g.nbx), p0, p1, ddy * ddy + ddz * ddz);
}

// One view's back-projection term of one voxel, added to capL (and, for the
// OS-SART kinds, the sensitivity): the tap pair (c, c + 1) x rows (r, r + 1)
// of its table entries ex, ey on the view's h section p, off-detector taps
// weighted 0 and their loads kept in bounds by the tables.
template <int KIND>
__device__ __forceinline__ void bp_view(const float* __restrict__ p, const float4 ex,
                                        const float4 ey, float s2, const nr_geom& g, float& capL,
                                        float& sens) {
    const float dw = __fdividef(s2, ex.w + ey.w);
    const float* q0 = p + (__float_as_int(ey.x) + __float_as_int(ex.x));
    const float* q1 = q0 + g.nbx;
    float d1 = ex.y * __ldg(q0);
    d1 = d1 + ex.z * __ldg(q0 + 1);
    float d2 = ex.y * __ldg(q1);
    d2 = d2 + ex.z * __ldg(q1 + 1);
    capL = capL + (ey.y * d1 + ey.z * d2) * g.vz * dw;
    if (KIND != UPD_OSTR) {  // sensitivity: the same weights on ones
        const float s1 = ex.y + ex.z;
        sens = sens + (ey.y * s1 + ey.z * s1) * g.vz * dw;
    }
}

// The update of one voxel from its sums, stored at out (non-finite values
// flagged in status).
template <int KIND>
__device__ __forceinline__ void upd_store(float xc, float capL, float sens, float rd, float rdd,
                                          float dv, float M, float beta, float* __restrict__ out,
                                          int* __restrict__ status) {
    float xn;
    if (KIND == UPD_OSTR) {
        capL = M * capL;
        xn = xc - __fdividef(capL + beta * rd, dv + 2.f * beta * rdd);
    } else {
        // Tomo_OSTR.cu:2193-2205: u/sens and beta*prior/sens, 0 without sensitivity
        float ut = 0.f, bt = 0.f;
        if (sens != 0.f) {
            ut = __fdiv_rn(capL, sens);
            if (KIND == UPD_SART_R) bt = __fdiv_rn(beta * rd, sens);
        }
        xn = xc + M * (ut + bt);
    }
    if (!(fabsf(xn) < __int_as_float(0x7f800000))) atomicOr(status, NR_FLAG_NONFINITE);
    *out = xn < 0.f ? 0.f : xn;
}

// One sub-iteration's update, fused: SBP of h (subset views, [view][j][i]),
// the penalty, and the update_est step.  Each block owns a 32 x 8 tile of
// (x, y) columns and walks UZC planes in z, keeping planes z-1, z, z+1 of x
// (with halo) in a 3-slot shared-memory ring, so every neighbour read is a
// shared-memory load at a fixed offset.  The global loads of plane z+2 are
// issued before plane z is computed (register prefetch), so they overlap the
// arithmetic.  The back projection reads the separable tables (BpTab).
// Writes x_out; flags non-finite values.
//
// KIND = UPD_SART / UPD_SART_R turn the same tile into the OS-SART update:
// h is the normalised projection difference of the subset, the back
// projection also sums the interpolation weights (the sensitivity), and
//     x' = max(0, x + lambda (sum_u + beta RD) / sum_sens)   (0 where sum_sens = 0)
// with lambda passed in M, RD the hyperbola gradient of x with unit
// neighbour distances (G_Huber_prior, Tomo_OSTR.cu:258-325; W built with
// z ratio 1) for UPD_SART_R, and d unused.
//
// NV > 0 fixes the subset's view count at compile time (nv is then NV): with
// one view per subset the per-view loop disappears, which saves ~40
// instructions per voxel and 8 registers.
template <int POT, int ZC = UZC, int KIND = UPD_OSTR, int NV = 0>
__device__ __forceinline__ void update_tile(
    const Geo& G, const PriorW5& W, const float* __restrict__ x, float* __restrict__ x_out,
    const float* __restrict__ d, const float* __restrict__ h, const float* __restrict__ angles,
    const int32_t* __restrict__ index, const BpTab& T, int a0, int nv, float M, float beta,
    float delta, int* __restrict__ status, int bx, int by, int bz, UpdSmem& sm) {
    float (*tile)[UPLANE] = sm.tile;
    ViewSrc* sv = sm.sv;
    const nr_geom& g = G.g;
    const int tid = threadIdx.y * UTX + threadIdx.x;
    for (int t = tid; t < (NV ? NV : nv); t += UTX * UTY)
        sv[t] = view_source(g, angles[index[a0 + t]]);
    const int x0t = bx * UTX, y0t = by * UTY;
    const int zb = bz * ZC, ze = min(zb + ZC, g.nz);
    // voxel and table indices in 32 bits: volumes hold fewer than 2^31 voxels
    // (geom_ok) and the tables fewer than 2^31 entries (bp_tables_fit)
    const int plane = g.nx * g.ny;
    // This thread's (at most two) cells of a halo plane tile.
    constexpr int NT = UTX * UTY;
    static_assert(UPLANE <= 2 * NT, "two cells per thread");
    const int e1 = tid + NT;
    const bool has1 = e1 < UPLANE;
    auto cell_off = [&](int k, bool& ok) -> int {
        const int r = k / USW, c = k - r * USW;
        const int gx = x0t - 1 + c, gy = y0t - 1 + r;
        ok = gx >= 0 && gx < g.nx && gy >= 0 && gy < g.ny;
        return ok ? gy * g.nx + gx : 0;
    };
    bool ok0, ok1 = false;
    const int off0 = cell_off(tid, ok0);
    const int off1 = has1 ? cell_off(e1, ok1) : 0;
    const float qnan = __int_as_float(0x7fc00000);  // outside the volume
    auto fetch = [&](int z, float& v0, float& v1) {
        const bool zin = z >= 0 && z < g.nz;
        v0 = (zin && ok0) ? __ldg(x + (z * plane + off0)) : qnan;
        v1 = (zin && ok1) ? __ldg(x + (z * plane + off1)) : qnan;
    };
    float* pb = tile[0];
    float* pc = tile[1];
    float* pa = tile[2];
    {
        float v0, v1;
        fetch(zb - 1, v0, v1);
        pb[tid] = v0;
        if (has1) pb[e1] = v1;
        fetch(zb, v0, v1);
        pc[tid] = v0;
        if (has1) pc[e1] = v1;
    }
    float n0, n1;
    fetch(zb + 1, n0, n1);
    const int ix = x0t + threadIdx.x, iy = y0t + threadIdx.y;
    const bool active = ix < g.nx && iy < g.ny;
    const bool edge_xy = x0t == 0 || x0t + UTX >= g.nx || y0t == 0 || y0t + UTY >= g.ny;
    const float inv_delta = 1.f / delta;
    const int64_t B = (int64_t)g.nbx * g.nby;
    const int r = threadIdx.y + 1, c = threadIdx.x + 1;
    for (int z = zb; z < ze; z++) {
        pa[tid] = n0;
        if (has1) pa[e1] = n1;
        __syncthreads();
        if (z + 1 < ze) fetch(z + 2, n0, n1);
        if (active) {
            const int v = z * plane + iy * g.nx + ix;
            const float dv = KIND == UPD_OSTR ? __ldg(d + v) : 0.f;
            const float xc = pc[r * USW + c];
            // M * SBP(h) from the plane's tables: the taps and weights of
            // bp.cu's sbp_term on the [j][i] layout.
            float capL = 0.f, sens = 0.f;
            const float* p = h;
            int tix = (a0 * g.nz + z) * g.nx + ix;
            int tiy = (a0 * g.nz + z) * g.ny + iy;
            const int sx = g.nz * g.nx, sy = g.nz * g.ny;
            for (int t = 0; t < (NV ? NV : nv); t++, p += B, tix += sx, tiy += sy)
                bp_view<KIND>(p, __ldg(T.x + tix), __ldg(T.y + tiy), sv[t].s2, g, capL, sens);
            float rdd = 0.f, rd = 0.f;
            const int base = r * USW + c;
            if (KIND != UPD_SART) {
                if (edge_xy || z == 0 || z == g.nz - 1)
                    prior_pairs<POT, true>(pb, pc, pa, base, xc, W, delta, inv_delta, &rdd, &rd);
                else
                    prior_pairs<POT, false>(pb, pc, pa, base, xc, W, delta, inv_delta, &rdd, &rd);
            }
            upd_store<KIND>(xc, capL, sens, rd, rdd, dv, M, beta, x_out + v, status);
        }
        __syncthreads();
        float* t = pb;
        pb = pc;
        pc = pa;
        pa = t;
    }
}

// ---- Two voxels per thread ----------------------------------------------
// The x2 tile: 64 x 8 columns, thread (tx, ty) owning voxels x0 + 2 tx and
// x0 + 2 tx + 1 of row y0 + ty.  The neighbour terms of its two voxels at one
// offset form a packed pair whose operands lie side by side in shared
// memory, so one 64-bit load brings both.  In a plane row with its halo the
// two voxels sit at cells 2 tx + 1 and 2 tx + 2: the dx = -1 and dx = +1
// pairs start at the even cells 2 tx and 2 tx + 2; the dx = 0 pairs (odd
// start) are read from a second copy of the plane stored one float later.
// Per voxel this halves the shared-memory loads of the penalty and shares
// the row table entry of the back projection.
constexpr int U2X = 2 * UTX;           // 64 columns
constexpr int U2W = U2X + 2;           // cells per row with the halo (even)
constexpr int U2PLANE = U2W * USH;     // cells per plane
constexpr int U2COPY = U2PLANE + 2;    // floats per copy (the shifted copy ends one later)
static_assert(U2W % 2 == 0 && U2COPY % 2 == 0, "8-byte aligned rows and copies");

struct UpdSmem2 {
    alignas(16) float tile[3][2 * U2COPY];  // per ring slot: copy 0 (cell k at k), copy 1 (at k + 1)
    ViewSrc sv[UPD_VIEWS_SMEM];
};

// Neighbour K of both voxels (base: the first voxel's cell in copy 0).
template <int POT, bool EDGE, int K>
__device__ __forceinline__ void nb_x2(const float* __restrict__ pb, const float* __restrict__ pc,
                                      const float* __restrict__ pa, int base, f32x2 xc2,
                                      const PriorW5& W, float delta, float inv_delta, f32x2& sdd,
                                      f32x2& sd) {
    constexpr int dz = K / 9 - 1, dy = (K / 3) % 3 - 1, dx = K % 3 - 1;
    const float* pl = dz < 0 ? pb : (dz == 0 ? pc : pa);
    const int at = dx == 0 ? U2COPY + base + 1 + dy * U2W : base + dy * U2W + dx;
    const f32x2 n2 = *reinterpret_cast<const f32x2*>(pl + at);
    nb_terms<POT, EDGE, nb_class<K>()>(sub2(xc2, n2), W, delta, inv_delta, sdd, sd);
}

// The penalty sums of both voxels.  Each voxel's neighbours are summed in
// the order and grouping of prior_pairs (its two partial sums, then their
// sum), so every voxel gets the bits the one-voxel tile gives it.
template <int POT, bool EDGE>
__device__ __forceinline__ void prior_x2(const float* __restrict__ pb,
                                         const float* __restrict__ pc,
                                         const float* __restrict__ pa, int base, f32x2 xc2,
                                         const PriorW5& W, float delta, float inv_delta,
                                         f32x2& rdd2, f32x2& rd2) {
    const f32x2 zero = pk2(0.f, 0.f);
    f32x2 dda = zero, da = zero, ddb = zero, db = zero;
#define NR_X2(ka, kb)                                                              \
    nb_x2<POT, EDGE, ka>(pb, pc, pa, base, xc2, W, delta, inv_delta, dda, da);    \
    nb_x2<POT, EDGE, kb>(pb, pc, pa, base, xc2, W, delta, inv_delta, ddb, db)
    NR_X2(0, 2); NR_X2(3, 5); NR_X2(6, 8);
    NR_X2(9, 11); NR_X2(12, 14); NR_X2(15, 17);
    NR_X2(18, 20); NR_X2(21, 23); NR_X2(24, 26);
    NR_X2(1, 7); NR_X2(19, 25); NR_X2(4, 22); NR_X2(10, 16);
#undef NR_X2
    rdd2 = add2(dda, ddb);
    rd2 = add2(da, db);
}

// update_tile on the x2 tile: the same sums and update, bit for bit, for the
// two voxels of each thread.  A voxel past the volume's last column is
// computed from out-of-volume cells and not stored.
template <int POT, int ZC = UZC, int KIND = UPD_OSTR, int NV = 0>
__device__ __forceinline__ void update_tile_x2(
    const Geo& G, const PriorW5& W, const float* __restrict__ x, float* __restrict__ x_out,
    const float* __restrict__ d, const float* __restrict__ h, const float* __restrict__ angles,
    const int32_t* __restrict__ index, const BpTab& T, int a0, int nv, float M, float beta,
    float delta, int* __restrict__ status, int bx, int by, int bz, UpdSmem2& sm) {
    ViewSrc* sv = sm.sv;
    const nr_geom& g = G.g;
    const int tid = threadIdx.y * UTX + threadIdx.x;
    for (int t = tid; t < (NV ? NV : nv); t += UTX * UTY)
        sv[t] = view_source(g, angles[index[a0 + t]]);
    const int x0t = bx * U2X, y0t = by * UTY;
    const int zb = bz * ZC, ze = min(zb + ZC, g.nz);
    const int plane = g.nx * g.ny;
    // This thread's (two or three) cells of a halo plane tile.
    constexpr int NT = UTX * UTY;
    static_assert(2 * NT <= U2PLANE && U2PLANE <= 3 * NT, "two or three cells per thread");
    const int e1 = tid + NT, e2 = tid + 2 * NT;
    const bool has2 = e2 < U2PLANE;
    auto cell_off = [&](int k, bool& ok) -> int {
        const int r = k / U2W, c = k - r * U2W;
        const int gx = x0t - 1 + c, gy = y0t - 1 + r;
        ok = gx >= 0 && gx < g.nx && gy >= 0 && gy < g.ny;
        return ok ? gy * g.nx + gx : 0;
    };
    bool ok0, ok1, ok2 = false;
    const int off0 = cell_off(tid, ok0);
    const int off1 = cell_off(e1, ok1);
    const int off2 = has2 ? cell_off(e2, ok2) : 0;
    const float qnan = __int_as_float(0x7fc00000);  // outside the volume
    auto fetch = [&](int z, float& v0, float& v1, float& v2) {
        const bool zin = z >= 0 && z < g.nz;
        v0 = (zin && ok0) ? __ldg(x + (z * plane + off0)) : qnan;
        v1 = (zin && ok1) ? __ldg(x + (z * plane + off1)) : qnan;
        v2 = (zin && ok2) ? __ldg(x + (z * plane + off2)) : qnan;
    };
    auto put = [&](float* pl, float v0, float v1, float v2) {
        pl[tid] = v0;
        pl[U2COPY + tid + 1] = v0;
        pl[e1] = v1;
        pl[U2COPY + e1 + 1] = v1;
        if (has2) {
            pl[e2] = v2;
            pl[U2COPY + e2 + 1] = v2;
        }
    };
    float* pb = sm.tile[0];
    float* pc = sm.tile[1];
    float* pa = sm.tile[2];
    float n0, n1, n2;
    fetch(zb - 1, n0, n1, n2);
    put(pb, n0, n1, n2);
    fetch(zb, n0, n1, n2);
    put(pc, n0, n1, n2);
    fetch(zb + 1, n0, n1, n2);
    const int ix = x0t + 2 * threadIdx.x, iy = y0t + threadIdx.y;
    const bool active = ix < g.nx && iy < g.ny;
    const bool has_b = ix + 1 < g.nx;   // the second voxel is in the volume
    const bool edge_xy = x0t == 0 || x0t + U2X >= g.nx || y0t == 0 || y0t + UTY >= g.ny;
    const float inv_delta = 1.f / delta;
    const int64_t B = (int64_t)g.nbx * g.nby;
    const int base = (threadIdx.y + 1) * U2W + 2 * threadIdx.x + 1;
    for (int z = zb; z < ze; z++) {
        put(pa, n0, n1, n2);
        __syncthreads();
        if (z + 1 < ze) fetch(z + 2, n0, n1, n2);
        if (active) {
            const int v = z * plane + iy * g.nx + ix;
            const float dva = KIND == UPD_OSTR ? __ldg(d + v) : 0.f;
            const float dvb = (KIND == UPD_OSTR && has_b) ? __ldg(d + v + 1) : 0.f;
            const f32x2 xc2 = *reinterpret_cast<const f32x2*>(pc + U2COPY + base + 1);
            float capa = 0.f, capb = 0.f, sensa = 0.f, sensb = 0.f;
            const float* p = h;
            int tix = (a0 * g.nz + z) * g.nx + ix;
            int tiy = (a0 * g.nz + z) * g.ny + iy;
            const int sx = g.nz * g.nx, sy = g.nz * g.ny;
            const int db = has_b ? 1 : 0;   // the second voxel's column entry (kept in bounds)
            for (int t = 0; t < (NV ? NV : nv); t++, p += B, tix += sx, tiy += sy) {
                const float4 ey = __ldg(T.y + tiy);
                const float s2 = sv[t].s2;
                bp_view<KIND>(p, __ldg(T.x + tix), ey, s2, g, capa, sensa);
                bp_view<KIND>(p, __ldg(T.x + tix + db), ey, s2, g, capb, sensb);
            }
            f32x2 rdd2 = pk2(0.f, 0.f), rd2 = pk2(0.f, 0.f);
            if (KIND != UPD_SART) {
                if (edge_xy || z == 0 || z == g.nz - 1)
                    prior_x2<POT, true>(pb, pc, pa, base, xc2, W, delta, inv_delta, rdd2, rd2);
                else
                    prior_x2<POT, false>(pb, pc, pa, base, xc2, W, delta, inv_delta, rdd2, rd2);
            }
            float xa, xb, rdda, rddb, rda, rdb;
            upk2(xc2, xa, xb);
            upk2(rdd2, rdda, rddb);
            upk2(rd2, rda, rdb);
            upd_store<KIND>(xa, capa, sensa, rda, rdda, dva, M, beta, x_out + v, status);
            if (has_b)
                upd_store<KIND>(xb, capb, sensb, rdb, rddb, dvb, M, beta, x_out + v + 1, status);
        }
        __syncthreads();
        float* t = pb;
        pb = pc;
        pc = pa;
        pa = t;
    }
}

// One block per (x, y) tile and chunk of ZC planes; NV as in update_tile.
// One-view kernels are held to 32 registers (8 resident blocks per SM: the
// paired prior would otherwise take 35-38).  The others carry no block
// minimum (40-44 registers, no spills); a minimum of 1 lets ptxas take 80-119
// and one of 5 spills 80 bytes.
template <int POT, int ZC, int NV>
__global__ void __launch_bounds__(256, NV == 1 ? 8 : 0) update_kernel(
    const __grid_constant__ Geo G, const __grid_constant__ PriorW5 W,
    const float* __restrict__ x, float* __restrict__ x_out, const float* __restrict__ d,
    const float* __restrict__ h, const float* __restrict__ angles,
    const int32_t* __restrict__ index, const __grid_constant__ BpTab T, int a0, int nv,
    float M, float beta, float delta, int* __restrict__ status) {
    __shared__ UpdSmem sm;
    update_tile<POT, ZC, UPD_OSTR, NV>(G, W, x, x_out, d, h, angles, index, T, a0, nv, M, beta,
                                       delta, status, blockIdx.x, blockIdx.y, blockIdx.z, sm);
}

// The same update on x2 tiles (64 x 8 columns per block), five resident
// blocks per SM (48 registers, no spills).  Measured per 25 updates at 16
// planes, clinical / full resolution: 5 blocks 6.54 / 17.42 ms, 6 blocks (40
// registers) 6.71 / 17.46 ms, 4 blocks (64 registers) 6.82 / 18.51 ms; held
// to 8 blocks (32 registers) it spills 20 bytes (0.275 ms per update).
template <int POT, int ZC, int NV>
__global__ void __launch_bounds__(256, NV == 1 ? 5 : 0) update_x2_kernel(
    const __grid_constant__ Geo G, const __grid_constant__ PriorW5 W,
    const float* __restrict__ x, float* __restrict__ x_out, const float* __restrict__ d,
    const float* __restrict__ h, const float* __restrict__ angles,
    const int32_t* __restrict__ index, const __grid_constant__ BpTab T, int a0, int nv,
    float M, float beta, float delta, int* __restrict__ status) {
    __shared__ UpdSmem2 sm;
    update_tile_x2<POT, ZC, UPD_OSTR, NV>(G, W, x, x_out, d, h, angles, index, T, a0, nv, M,
                                          beta, delta, status, blockIdx.x, blockIdx.y,
                                          blockIdx.z, sm);
}


// ---- TMA-fed ring -----------------------------------------------------------
// The one-voxel tile with its planes streamed by TMA instead of through the
// threads' registers: lane 0 of warp 0 loads each plane of the tile with its
// halo (one cp.async.bulk.tensor.3d box of UTW x USH voxels starting 4 voxels
// left of the tile, so that the box's x coordinate is a multiple of 4 floats;
// out-of-volume voxels read as NaN, the ring's convention for "outside") into
// a ring of UT_SLOTS slots, each with a "full" mbarrier (the copy landed) and
// an "empty" one (all eight warps are done with the plane).  Each warp runs
// update_tile's arithmetic on its row of the tile, plane by plane, waiting
// only for the plane it needs next: there is no block-wide barrier per
// plane, so a warp held up by its back-projection loads does not hold the
// others up, and up to UT_SLOTS - 3 planes are in flight ahead of the
// slowest warp.  Warp 0 refills a slot once every warp is done with it.
// Results are bit-identical to update_tile's (same sums in the same order).
//
// Every wait is bounded.  A wait that gives up flags NR_FLAG_TIMEOUT, after
// which that thread waits no more (the tile's output is then not to be
// used; the host reads the flag as NR_ERR_TIMEOUT).  Once the issuing lane
// has given up it issues no further copy, so no slot whose readers are
// unaccounted for is refilled, and before it exits it waits (bounded) for
// every copy it issued, so none is in flight when the block's shared memory
// is released.  A first version with a ninth, producer-only warp held 7
// blocks per SM instead of 8 and ran 11 % slower on the clinical workload.
constexpr int UTW = UTX + 8;            // columns of a staged row: x0 - 4 .. x0 + 35
constexpr int UT_SLOT = 416;            // floats per slot: UTW x USH = 400, rounded to 128 B
constexpr int UT_SLOTS = 6;
constexpr uint32_t UT_BYTES = UTW * USH * 4;
constexpr int UT_WAIT = 1 << 22;        // polls before a wait gives up
static_assert(UTW * USH <= UT_SLOT && (UT_SLOT * 4) % 128 == 0, "slot size");

struct UpdSmemT {
    alignas(128) float ring[UT_SLOTS][UT_SLOT];
    alignas(8) uint64_t full[UT_SLOTS];
    uint64_t empty[UT_SLOTS];
    ViewSrc sv[UPD_VIEWS_SMEM];
};

template <int POT, int ZC = UZC, int KIND = UPD_OSTR, int NV = 0>
__device__ __forceinline__ void update_tile_tma(
    const Geo& G, const PriorW5& W, const CUtensorMap* map, float* __restrict__ x_out,
    const float* __restrict__ d, const float* __restrict__ h, const float* __restrict__ angles,
    const int32_t* __restrict__ index, const BpTab& T, int a0, int nv, float M, float beta,
    float delta, int* __restrict__ status, int bx, int by, int bz, UpdSmemT& sm) {
    const nr_geom& g = G.g;
    const int warp = threadIdx.y, lane = threadIdx.x;
    const int tid = warp * UTX + lane;
    for (int t = tid; t < (NV ? NV : nv); t += UTX * UTY)
        sm.sv[t] = view_source(g, angles[index[a0 + t]]);
    const int x0t = bx * UTX, y0t = by * UTY;
    const int zb = bz * ZC, ze = min(zb + ZC, g.nz);
    const int np = ze - zb + 2;  // planes zb - 1 .. ze; plane k is z = zb - 1 + k
    const bool issuer = tid == 0;
    bool issuing = true;         // the issuer: false once one of its waits gave up
    int issued = np;             // planes issued: all of them unless the issuer gave up
    auto issue = [&](int k, int s) {  // plane k into slot s = k % UT_SLOTS (its last reader done)
        tc::fence_async_smem();
        mbar_arrive_tx(&sm.full[s], UT_BYTES);
        tma_load_3d(&sm.ring[s][0], map, x0t - 4, y0t - 1, zb - 1 + k, &sm.full[s]);
    };
    if (issuer) {
        for (int s = 0; s < UT_SLOTS; s++) {
            tc::mbar_init(&sm.full[s], 1);
            tc::mbar_init(&sm.empty[s], UTY);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int k = 0; k < min(np, UT_SLOTS); k++) issue(k, k);
    }
    __syncthreads();
    bool live = true;  // false after a wait of this thread gave up: it waits no more
    // test hook: the workspace's second status word k + 1 > 0 makes the wait
    // for plane k report giving up once it has in fact succeeded
    const int force_at = status[1] - 1;
    auto wait_full = [&](int k, int s, uint32_t parity) {  // plane k, in slot s
        if (live && (!tc::mbar_wait(&sm.full[s], parity, UT_WAIT) || k == force_at)) {
            if (lane == 0) atomicOr(status, NR_FLAG_TIMEOUT);
            live = false;
        }
    };
    const int ix = x0t + lane, iy = y0t + warp;
    const bool active = ix < g.nx && iy < g.ny;
    const bool edge_xy = x0t == 0 || x0t + UTX >= g.nx || y0t == 0 || y0t + UTY >= g.ny;
    const float inv_delta = 1.f / delta;
    const int plane = g.nx * g.ny;
    const int64_t B = (int64_t)g.nbx * g.nby;
    const int base = (warp + 1) * UTW + lane + 4;
    // ring slot and barrier parity of planes k - 1, k and k + 1, carried from
    // plane to plane (slot p % UT_SLOTS, parity (p / UT_SLOTS) & 1 of plane p)
    int sb = 0, sc = 1, sa = 2;
    uint32_t qb = 0, qa = 0;
    static_assert(UT_SLOTS > 3, "planes 0..2 share the first pass of the ring");
    wait_full(0, 0, 0);
    wait_full(1, 1, 0);
    for (int z = zb; z < ze; z++) {
        const int k = z - zb + 1;  // the centre plane's ring index
        wait_full(k + 1, sa, qa);
        const float* pb = sm.ring[sb];
        const float* pc = sm.ring[sc];
        const float* pa = sm.ring[sa];
        if (active) {
            const int v = z * plane + iy * g.nx + ix;
            const float dv = KIND == UPD_OSTR ? __ldg(d + v) : 0.f;
            const float xc = pc[base];
            float capL = 0.f, sens = 0.f;
            const float* p = h;
            int tix = (a0 * g.nz + z) * g.nx + ix;
            int tiy = (a0 * g.nz + z) * g.ny + iy;
            const int sx = g.nz * g.nx, sy = g.nz * g.ny;
            for (int t = 0; t < (NV ? NV : nv); t++, p += B, tix += sx, tiy += sy)
                bp_view<KIND>(p, __ldg(T.x + tix), __ldg(T.y + tiy), sm.sv[t].s2, g, capL, sens);
            float rdd = 0.f, rd = 0.f;
            if (KIND != UPD_SART) {
                if (edge_xy || z == 0 || z == g.nz - 1)
                    prior_pairs_w<POT, true, UTW>(pb, pc, pa, base, xc, W, delta, inv_delta, &rdd,
                                                  &rd);
                else
                    prior_pairs_w<POT, false, UTW>(pb, pc, pa, base, xc, W, delta, inv_delta,
                                                   &rdd, &rd);
            }
            upd_store<KIND>(xc, capL, sens, rd, rdd, dv, M, beta, x_out + v, status);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.empty[sb]);
        // plane k - 1 + UT_SLOTS goes where plane k - 1 was, once every warp is done with it
        const int kn = k - 1 + UT_SLOTS;
        if (issuer && issuing && kn < np) {
            if (tc::mbar_wait(&sm.empty[sb], qb, UT_WAIT)) {
                issue(kn, sb);
            } else {
                atomicOr(status, NR_FLAG_TIMEOUT);
                issuing = false;
                issued = kn;
            }
        }
        // rotate: k - 1 <- k, k <- k + 1, k + 1 <- k + 2
        qb = (sc < sb) ? qb ^ 1u : qb;  // plane k's parity: plane k - 1's, flipped on a wrap
        sb = sc;
        sc = sa;
        if (++sa == UT_SLOTS) {
            sa = 0;
            qa ^= 1u;
        }
    }
    if (issuer) {
        // no copy may be in flight when the block exits
        for (int k = max(0, issued - UT_SLOTS); k < issued; k++) {
            const int s = k % UT_SLOTS;
            if (!tc::mbar_wait(&sm.full[s], (k / UT_SLOTS) & 1, UT_WAIT)) {
                atomicOr(status, NR_FLAG_TIMEOUT);
                tc::mbar_wait(&sm.full[s], (k / UT_SLOTS) & 1, UT_WAIT);
            }
        }
    }
}

// One block per (x, y) tile and chunk of ZC planes, 8 warps (one row each);
// one-view kernels held to 32 registers (8 resident blocks per SM).
template <int POT, int ZC, int NV>
__global__ void __launch_bounds__(256, NV == 1 ? 8 : 0) update_tma_kernel(
    const __grid_constant__ Geo G, const __grid_constant__ PriorW5 W,
    const __grid_constant__ CUtensorMap map, float* __restrict__ x_out,
    const float* __restrict__ d, const float* __restrict__ h, const float* __restrict__ angles,
    const int32_t* __restrict__ index, const __grid_constant__ BpTab T, int a0, int nv,
    float M, float beta, float delta, int* __restrict__ status) {
    __shared__ UpdSmemT sm;
    update_tile_tma<POT, ZC, UPD_OSTR, NV>(G, W, &map, x_out, d, h, angles, index, T, a0, nv, M,
                                           beta, delta, status, blockIdx.x, blockIdx.y,
                                           blockIdx.z, sm);
}

}  // namespace nr
