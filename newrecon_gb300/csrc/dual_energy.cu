// dual_energy.cu -- weighted dual-energy subtraction of two reconstructions.
//
// syncrecon.m (the reference's post-processing of a high- and a low-energy
// OSTR volume) forms, for every weight w of a list, d = he - le * w and writes
// d as float32; it prints the entropy of one slice of each d, and computes an
// Otsu threshold of he (graythresh) whose mask it applies in commented-out
// lines.  MATLAB reads the float32 files as double, so d is
//     float(double(he) - double(le) * w)        (two roundings in double)
// which the kernel reproduces bit for bit: in FP32 by error-free transforms
// where a bound on what they drop decides the rounding (de_fast), and with
// separate double multiply and subtract (no contraction to an FMA) where it
// cannot -- GB300's FP64 pipe runs at about 1/64 of the FP32 rate.  The K
// outputs of one voxel are written from one read of he and le.
//
// Image-statistics helpers (the 8-bit conversion of MATLAB's entropy and
// graythresh): a value v maps to bin round(255 v) (half away from zero),
// saturated to [0, 255], NaN to 0.
#include <cmath>

#include "common.cuh"

namespace nr {

constexpr int DE_MAX_WEIGHTS = 16;

struct DeWeights {
    double w[DE_MAX_WEIGHTS];
    float w1[DE_MAX_WEIGHTS], w2[DE_MAX_WEIGHTS];  // w = w1 + w2 + (|.| <= 2^-47 |w|)
    unsigned fast;     // bit k: weight k takes the FP32 path (de_fast)
    unsigned pow2;     // bit k: weight k is a power of two (a w exact in float)
    int k;
    int masked;        // 1: he and le multiplied by (he > level) first
    double level;
    float level_f;     // the largest float <= level: (double)h > level iff h > level_f
};

__device__ __forceinline__ int im8_bin(double v) {
    if (!(v == v)) return 0;
    const double r = round(255.0 * v);   // CUDA round(): half away from zero
    return r <= 0.0 ? 0 : (r >= 255.0 ? 255 : (int)r);
}

__device__ __forceinline__ double de_value(double h, double l, double w) {
    return __dadd_rn(h, -__dmul_rn(l, w));
}

// float(double(b) - double(a) * w) without the FP64 pipe, or NaN when the
// FP32 evaluation cannot decide it (the caller then takes the FP64 path).
//
// a w1 = p1 + e1 exactly (FMA), a w2 rounds once; two error-free sums give
// b - a w ~ hi + lo with hi = RN(hi + lo).  The terms dropped on the way (a
// w2's rounding and the w tail, under 2^-47 |p1|; the float sums of the
// small terms, under 2^-48 (2 |s| + 3 |p1|), s = RN(b - p1)) and both
// roundings of the double evaluation (under 2^-53 (|b| + 2 |p1|)) add up to
// less than 2^-45.2 |p1| + 2^-46.9 |b|; B = 2^-44 |p1| + 2^-46 |b| bounds
// them with a factor of 1.8 to spare.  If hi + m and hi - m, m = |lo| + B,
// both round back to hi, the double evaluation lies strictly inside hi's
// rounding interval and rounds to hi too.  Otherwise -- about 2^-20 |p1| /
// |hi| of the outputs (cancellation), and tiny, huge or non-finite products
// -- the answer is left to FP64.
// b - a w ~ hi + lo as above, with B bounding |the double value - (hi + lo)|;
// false for tiny, huge or non-finite products.
__device__ __forceinline__ bool de_sum(float b, float a, float w1, float w2, float& hi, float& lo,
                                       float& B) {
    const float p1 = __fmul_rn(a, w1);
    const float ap1 = fabsf(p1);
    if (!(ap1 >= 0x1p-100f && ap1 <= 0x1p100f)) return false;
    const float e1 = __fmaf_rn(a, w1, -p1);
    const float q = __fmul_rn(a, w2);
    const float s = __fsub_rn(b, p1);  // TwoSum(b, -p1)
    const float bp = __fsub_rn(s, b);
    const float ap = __fsub_rn(s, bp);
    const float serr = __fsub_rn(__fsub_rn(b, ap), __fadd_rn(p1, bp));
    const float t = __fsub_rn(__fsub_rn(serr, e1), q);
    hi = __fadd_rn(s, t);  // TwoSum(s, t)
    const float tp = __fsub_rn(hi, s);
    const float sp = __fsub_rn(hi, tp);
    lo = __fadd_rn(__fsub_rn(s, sp), __fsub_rn(t, tp));
    B = __fmaf_rn(fabsf(b), 0x1p-46f, __fmul_rn(ap1, 0x1p-44f));
    return true;
}

__device__ __forceinline__ float de_fast(float b, float a, float w1, float w2) {
    float hi, lo, B;
    if (de_sum(b, a, w1, w2, hi, lo, B)) {
        const float m = __fadd_rn(fabsf(lo), B);
        if (__fadd_rn(hi, m) == hi && __fsub_rn(hi, m) == hi) return hi;
    }
    return __int_as_float(0x7fc00000);
}

// im8_bin of a double value v known as |v - (hi + lo)| <= B: round(255 v)
// half away from zero, saturated to [0, 255]; -1 when v lies too close to a
// bin edge (255 v = k + 1/2) for the float evaluation to tell.
__device__ __forceinline__ int de_bin(float hi, float lo, float B) {
    const float yh = __fmul_rn(255.f, hi);
    const float ye = __fmaf_rn(255.f, hi, -yh);  // exact
    const float y = __fadd_rn(yh, __fmaf_rn(255.f, lo, ye));
    const float err = __fmaf_rn(255.f, B, __fmaf_rn(fabsf(y), 0x1p-22f, 0x1p-40f));
    const float f = floorf(__fadd_rn(y, 0.5f));
    const float dist = __fsub_rn(0.5f, fabsf(__fsub_rn(y, f)));
    if (!(dist > err)) return -1;  // also NaN
    return f <= 0.f ? 0 : (f >= 255.f ? 255 : (int)f);
}

// The FP64 evaluation, out of line: inlined, ptxas predicates it and runs
// it for every output beside the FP32 one.
__device__ __noinline__ float de_slow(float b, float a, double w) {
    return __double2float_rn(de_value(b, a, w));
}

template <int K>
__device__ __forceinline__ float de_out(float b, float a, const DeWeights& W) {
    if ((W.pow2 >> K) & 1u) {
        // a w exact: double(b) - a w needs more than 53 bits only when one
        // operand is below 2^-29 of the other, and then both roundings land
        // on the float of b - a w (the nearest float midpoint is 2^-25 away)
        const float p = __fmul_rn(a, W.w1[K]);
        const float ap = fabsf(p);
        if (a == 0.f || (ap >= 0x1p-100f && ap <= 0x1p100f)) return __fsub_rn(b, p);
    } else if ((W.fast >> K) & 1u) {
        const float r = de_fast(b, a, W.w1[K], W.w2[K]);
        if (r == r) return r;
        // a = 0 is exact in float: b - 0 w1, with IEEE's signed zeros as in double
        if (a == 0.f) return __fsub_rn(b, __fmul_rn(a, W.w1[K]));
    }
    return de_slow(b, a, W.w[K]);
}

// Weights K, K + 1, ... of four voxels (16-byte store per weight) or of one.
template <int K>
__device__ __forceinline__ void de_row(const float (&h)[4], const float (&l)[4],
                                       const DeWeights& W, float* __restrict__ d, int64_t n,
                                       int64_t q) {
    if constexpr (K < DE_MAX_WEIGHTS) {
        if (K >= W.k) return;
        float4 o;
        o.x = de_out<K>(h[0], l[0], W);
        o.y = de_out<K>(h[1], l[1], W);
        o.z = de_out<K>(h[2], l[2], W);
        o.w = de_out<K>(h[3], l[3], W);
        __stcs(reinterpret_cast<float4*>(d + (int64_t)K * n) + q, o);
        de_row<K + 1>(h, l, W, d, n, q);
    }
}

template <int K>
__device__ __forceinline__ void de_one(float h, float l, const DeWeights& W,
                                       float* __restrict__ d, int64_t n, int64_t i) {
    if constexpr (K < DE_MAX_WEIGHTS) {
        if (K >= W.k) return;
        d[(int64_t)K * n + i] = de_out<K>(h, l, W);
        de_one<K + 1>(h, l, W, d, n, i);
    }
}

// d[k][i] = float(he[i] - le[i] * w_k).  VEC (n a multiple of 4, so that every
// output row d + k n stays 16-byte aligned): four voxels per thread per step
// with 16-byte loads and stores; otherwise one voxel per step.
template <bool VEC>
__global__ void __launch_bounds__(256) de_subtract_kernel(const float* __restrict__ he,
                                                          const float* __restrict__ le,
                                                          float* __restrict__ d, int64_t n,
                                                          const __grid_constant__ DeWeights W) {
    const int64_t n4 = VEC ? n / 4 : 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += stride) {
        const float4 h4 = __ldg(reinterpret_cast<const float4*>(he) + q);
        const float4 l4 = __ldg(reinterpret_cast<const float4*>(le) + q);
        float h[4] = {h4.x, h4.y, h4.z, h4.w};
        float l[4] = {l4.x, l4.y, l4.z, l4.w};
        if (W.masked)
            for (int t = 0; t < 4; t++)
                if (!(h[t] > W.level_f)) h[t] = l[t] = 0.f;
        // unrolled over the weights: each weight's constants are fixed
        // constant-bank operands
        de_row<0>(h, l, W, d, n, q);
    }
    // everything when !VEC
    for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        float h = he[i], l = le[i];
        if (W.masked && !(h > W.level_f)) h = l = 0.f;
        de_one<0>(h, l, W, d, n, i);
    }
}

// hist[k][b] += voxels of [begin, begin + len) whose double d_k falls in bin
// b; the double value (before rounding to float) as MATLAB's entropy sees it.
__global__ void __launch_bounds__(256) de_hist_kernel(const float* __restrict__ he,
                                                      const float* __restrict__ le,
                                                      int64_t begin, int64_t len,
                                                      int* __restrict__ hist,
                                                      const __grid_constant__ DeWeights W) {
    __shared__ int sh[DE_MAX_WEIGHTS * 256];
    for (int t = threadIdx.x; t < W.k * 256; t += blockDim.x) sh[t] = 0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x) {
        float h = he[begin + i], l = le[begin + i];
        if (W.masked && !(h > W.level_f)) h = l = 0.f;
        for (int k = 0; k < W.k; k++) {
            int bin = -1;
            if ((W.fast >> k) & 1u) {
                float hi = h, lo = 0.f, B = 0.f;  // a = 0: the double value is b
                if (l == 0.f || de_sum(h, l, W.w1[k], W.w2[k], hi, lo, B)) bin = de_bin(hi, lo, B);
            }
            if (bin < 0) bin = im8_bin(de_value(h, l, W.w[k]));
            atomicAdd(&sh[k * 256 + bin], 1);
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < W.k * 256; t += blockDim.x)
        if (sh[t]) atomicAdd(&hist[t], sh[t]);
}

// hist[b] += voxels of x in bin b (graythresh's 8-bit histogram).
__global__ void __launch_bounds__(256) hist8_kernel(const float* __restrict__ x, int64_t n,
                                                    int* __restrict__ hist) {
    __shared__ int sh[256];
    sh[threadIdx.x] = 0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&sh[im8_bin((double)x[i])], 1);
    __syncthreads();
    if (sh[threadIdx.x]) atomicAdd(&hist[threadIdx.x], sh[threadIdx.x]);
}

static unsigned de_blocks(int64_t work) {
    int64_t b = (work + 255) / 256;
    return (unsigned)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

}  // namespace nr

using namespace nr;

NR_API nr_status nr_de_subtract(const float* he, const float* le, const double* weights,
                                int32_t n_weights, int64_t n, double mask_level, float* d,
                                int64_t hist_begin, int64_t hist_len, int32_t* hist,
                                void* stream) {
    if (!he || !le || !weights || !d || n < 0) return NR_ERR_BAD_ARGUMENT;
    if (n_weights < 1 || n_weights > DE_MAX_WEIGHTS) return NR_ERR_BAD_ARGUMENT;
    if (hist && (hist_begin < 0 || hist_len < 0 || hist_begin + hist_len > n))
        return NR_ERR_BAD_ARGUMENT;
    if (((uintptr_t)he | (uintptr_t)le | (uintptr_t)d) & 15) return NR_ERR_BAD_ARGUMENT;
    // float4 path: he, le, d 16-byte aligned (checked) and n % 4 == 0, so each
    // row d + k n is aligned too; q < n/4 keeps every access below n.
    DeWeights W;
    W.fast = 0u;
    W.pow2 = 0u;
    for (int k = 0; k < DE_MAX_WEIGHTS; k++) {
        const double w = k < n_weights ? weights[k] : 0.0;
        W.w[k] = w;
        // w = w1 + w2 + w3: both differences are exact in double
        const float w1 = (float)w;
        const float w2 = (float)(w - (double)w1);
        const double w3 = (w - (double)w1) - (double)w2;
        W.w1[k] = w1;
        W.w2[k] = w2;
        const double aw = std::fabs(w);
        if (k < n_weights && std::isfinite(w) && aw >= 0x1p-60 && aw <= 0x1p60 &&
            std::fabs(w3) <= std::ldexp(aw, -47))
            W.fast |= 1u << k;
        int ex = 0;
        if (k < n_weights && std::isfinite(w) && w != 0.0 && std::fabs(std::frexp(w, &ex)) == 0.5 &&
            ex > -90 && ex < 90)
            W.pow2 |= 1u << k;
    }
    W.k = n_weights;
    W.masked = mask_level >= 0.0;
    W.level = mask_level;
    float lf = (float)mask_level;
    if ((double)lf > mask_level) lf = std::nextafterf(lf, -INFINITY);
    W.level_f = lf;
    cudaStream_t s = as_stream(stream);
    if (n > 0 && n % 4 == 0)
        de_subtract_kernel<true><<<de_blocks(n / 4), 256, 0, s>>>(he, le, d, n, W);
    else if (n > 0)
        de_subtract_kernel<false><<<de_blocks(n), 256, 0, s>>>(he, le, d, n, W);
    if (hist) {
        if (cudaMemsetAsync(hist, 0, (size_t)n_weights * 256 * sizeof(int32_t), s) != cudaSuccess)
            return NR_ERR_CUDA;
        if (hist_len > 0)
            de_hist_kernel<<<de_blocks(hist_len), 256, 0, s>>>(he, le, hist_begin, hist_len,
                                                               hist, W);
    }
    return launch_status();
}

NR_API nr_status nr_hist8(const float* x, int64_t n, int32_t* hist, void* stream) {
    if (!x || !hist || n < 0) return NR_ERR_BAD_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    if (cudaMemsetAsync(hist, 0, 256 * sizeof(int32_t), s) != cudaSuccess) return NR_ERR_CUDA;
    if (n > 0) hist8_kernel<<<de_blocks(n), 256, 0, s>>>(x, n, hist);
    return launch_status();
}

// Host: Shannon entropy (bits) of a 256-bin histogram of `count` values,
// -sum p log2 p over the non-empty bins, p = hist / count.
NR_API nr_status nr_hist_entropy(const int32_t* hist, int64_t count, double* entropy) {
    if (!hist || !entropy || count <= 0) return NR_ERR_BAD_ARGUMENT;
    double e = 0.0;
    for (int b = 0; b < 256; b++) {
        if (hist[b] <= 0) continue;
        const double p = (double)hist[b] / (double)count;
        e -= p * std::log2(p);
    }
    *entropy = e;
    return NR_OK;
}

// Host: Otsu's threshold (Otsu 1979) of a 256-bin histogram: the bin k that
// maximises the between-class variance (mu_T w(k) - mu(k))^2 / (w(k)(1 - w(k))),
// w and mu the cumulative class probability and first moment; with several
// maxima the mean of their indices; returned as k / 255 (0 when the maximum is
// not finite, e.g. one occupied bin).
NR_API nr_status nr_otsu_level(const int32_t* hist, double* level) {
    if (!hist || !level) return NR_ERR_BAD_ARGUMENT;
    double total = 0.0;
    for (int b = 0; b < 256; b++) total += hist[b] > 0 ? (double)hist[b] : 0.0;
    if (!(total > 0.0)) return NR_ERR_BAD_ARGUMENT;
    double sb[256], w = 0.0, mu = 0.0, mu_t = 0.0;
    for (int b = 0; b < 256; b++) mu_t += (hist[b] > 0 ? hist[b] / total : 0.0) * (b + 1);
    double best = -1.0;
    for (int b = 0; b < 256; b++) {
        const double p = hist[b] > 0 ? hist[b] / total : 0.0;
        w += p;
        mu += p * (b + 1);
        const double num = mu_t * w - mu;
        sb[b] = num * num / (w * (1.0 - w));
        if (sb[b] > best) best = sb[b];   // NaN/inf never win: compared below
    }
    if (!(best >= 0.0) || !(best < INFINITY)) {
        *level = 0.0;
        return NR_OK;
    }
    double sum = 0.0;
    int cnt = 0;
    for (int b = 0; b < 256; b++)
        if (sb[b] == best) {
            sum += b + 1;
            cnt++;
        }
    *level = (sum / cnt - 1.0) / 255.0;
    return NR_OK;
}
