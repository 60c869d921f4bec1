// project.cuh -- the fused forward projection + OSTR gradient of one block of
// bins (device code shared by the single-reconstruction kernel in fp.cu and the
// batched kernel in batch.cu).
#pragma once

#include "reduce.cuh"
#include "siddon.cuh"

namespace nr {

// Detector offset of bin (i, j) of one view: JI -> [j][i] (i fastest, the
// layout of the fused path and of the scanner files); otherwise [i][j] (the
// reference's in-memory layout, Tomo_OSTR.cu:1365).
template <bool JI>
__device__ __forceinline__ int64_t bin_off(const nr_geom& g, int i, int j) {
    return JI ? (int64_t)j * g.nbx + i : (int64_t)i * g.nby + j;
}

// Fused forward projection + OSTR gradient h for the subset views of the
// device-resident path.  Detector arrays are [view][j][i] in subset order;
// y, b (and r) are indexed by the subset position a.  Rays that miss the
// volume have line = 0 (the reference zeroes the line buffer every subset,
// Tomo_OSTR_gold.cpp:843).  h = (y/(b e^-l + r) - 1) b e^-l,
// Tomo_OSTR_gold.cpp:245-260.
// One block of 32 x 4 bins (bx, by) of subset view bz.  Every thread of the
// block must call it (it synchronises once, twice with DATA).
//
// DATA: also the subset's FP64 data term, sum over its bins of
// ybar + r - y log(ybar + r) with ybar = b exp(-l) -- the data term of the
// objective (objective.cu) restricted to these views, each bin's term formed
// exactly as there -- as this block's partial in red[block] (warp shuffles,
// then a fixed-order block sum).
template <int K = 4, bool DATA = false>
__device__ __forceinline__ void fp_h_tile(const Geo& G, const float* __restrict__ vol,
                                          float* __restrict__ h, const float* __restrict__ angles,
                                          const int32_t* __restrict__ index, int a0,
                                          const float* __restrict__ y, const float* __restrict__ b,
                                          const float* __restrict__ r, int bx, int by, int bz,
                                          ViewSrc& src, double* __restrict__ red = nullptr) {
    const nr_geom& g = G.g;
    const int a = a0 + bz;
    if (threadIdx.x == 0 && threadIdx.y == 0) src = view_source(g, angles[index[a]]);
    __syncthreads();
    const int i = bx * 32 + threadIdx.x;
    const int j = by * 4 + threadIdx.y;
    const bool on = i < g.nbx && j < g.nby;
    if (!DATA && !on) return;
    double term = 0.0;
    if (on) {
        float v = 0.f;
        float l = 0.f;
        if (trace<0, K>(G, vol, src.x0, src.y0, src.z0, bin_x(g, i), bin_y(g, j), -g.detectorR,
                        &v))
            l = v * src.ct;
        const int64_t B = (int64_t)g.nbx * g.nby;
        const int64_t o = (int64_t)a * B + bin_off<true>(g, i, j);
        const float yb = b[o] * expf(-l);
        const float rr = r ? r[o] : 0.f;
        const float den = yb + rr;
        h[(int64_t)bz * B + bin_off<true>(g, i, j)] = (__fdiv_rn(y[o], den) - 1.f) * yb;
        if (DATA) {
            const double ybd = (double)b[o] * exp(-(double)l);
            const double m = ybd + (double)rr;
            const double yy = (double)y[o];
            term = m - (yy > 0.0 ? yy * log(m) : 0.0);
        }
    }
    if (DATA)
        block_partial(term, red, ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x +
                                     blockIdx.x);
}

}  // namespace nr
