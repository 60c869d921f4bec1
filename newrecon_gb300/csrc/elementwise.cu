// elementwise.cu -- the reference's per-bin / per-voxel host helpers, on the
// device (compute_yry, compute_gamma_yry, compute_h, update_est, the subset
// scaling, regroup_prj and x_y_flip of Tomo_OSTR_gold.cpp:93-295), plus the
// SART projection difference (Tomo_OSTR.cu:2145-2183) and log transform.
#include "common.cuh"

namespace nr {

__global__ void yry_kernel(float* __restrict__ yry, const float* __restrict__ prj,
                           const float* __restrict__ scat, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float y = prj[i];
        float out = 0.f;
        if (y != 0.f) {
            float dif = y - (scat ? scat[i] : 0.f);
            if (dif <= 0.f) dif = y;
            out = __fdiv_rn(dif * dif, y);
        }
        yry[i] = out;
    }
}

__global__ void mul_kernel(float* __restrict__ out, const float* __restrict__ a,
                           const float* __restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a[i] * b[i];
}

__global__ void h_kernel(float* __restrict__ h, const float* __restrict__ prj,
                         const float* __restrict__ blank, const float* __restrict__ line,
                         const float* __restrict__ scat, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float yb = blank[i] * expf(-line[i]);
        h[i] = (__fdiv_rn(prj[i], yb + (scat ? scat[i] : 0.f)) - 1.f) * yb;
    }
}

__global__ void update_est_kernel(float* __restrict__ est, const float* __restrict__ capL,
                                  const float* __restrict__ RD, const float* __restrict__ d,
                                  const float* __restrict__ RDD, float beta, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float v = est[i] - __fdiv_rn(capL[i] + beta * RD[i], d[i] + 2.f * beta * RDD[i]);
        est[i] = v < 0.f ? 0.f : v;
    }
}

// SART_prj_diff_kernel, Tomo_OSTR.cu:2145-2183: (prj - est) / normprj where
// normprj != 0, else 0.
__global__ void prj_diff_kernel(float* __restrict__ diff, const float* __restrict__ prj,
                                const float* __restrict__ est, const float* __restrict__ norm,
                                int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float nv = norm[i];
        diff[i] = nv != 0.f ? __fdiv_rn(prj[i] - est[i], nv) : 0.f;
    }
}

// Line integrals of a transmission scan for SART: log(blank / (prj - scat))
// where both are positive, else 0 (the log transform g = log I0 - log I of
// the reference's MATLAB examples, ReconDBT/gen_dbtproj_example.m:113).
__global__ void line_kernel(float* __restrict__ line, const float* __restrict__ prj,
                           const float* __restrict__ blank, const float* __restrict__ scat,
                           int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float nu = prj[i] - (scat ? scat[i] : 0.f);
        const float b = blank[i];
        line[i] = (nu > 0.f && b > 0.f) ? logf(__fdiv_rn(b, nu)) : 0.f;
    }
}

__global__ void scale_kernel(float* __restrict__ buf, float s, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        buf[i] = s * buf[i];
}

// out[v][b] = in[src(v)][b] where src is the regroup map; b contiguous.
__global__ void regroup_kernel(float* __restrict__ out, const float* __restrict__ in, int M,
                               int Vs, int64_t bsize) {
    const int v = blockIdx.y;              // output view = i*Vs + j
    const int i = v / Vs, j = v % Vs;
    const int src = j * M + i;
    const float* s = in + (int64_t)src * bsize;
    float* o = out + (int64_t)v * bsize;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < bsize;
         k += (int64_t)gridDim.x * blockDim.x)
        o[k] = s[k];
}

// Tiled transpose of each view: out[v][r][c] = in[v][c][r]; in is rows x cols.
// With view_map != nullptr, output view v takes input view view_map(v).
__global__ void transpose_kernel(float* __restrict__ out, const float* __restrict__ in, int rows,
                                 int cols, int M, int Vs) {
    __shared__ float tile[32][33];
    const int v = blockIdx.z;
    int src = v;
    if (M > 0) src = (v % Vs) * M + v / Vs;  // regrouped position v <- original view
    const float* s = in + (int64_t)src * rows * cols;
    float* o = out + (int64_t)v * rows * cols;
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = r0 + k, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[k][threadIdx.x] = s[(int64_t)r * cols + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = c0 + k, r = r0 + threadIdx.x;
        if (r < rows && c < cols) o[(int64_t)c * rows + r] = tile[threadIdx.x][k];
    }
}

static unsigned ew_blocks(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (unsigned)(b > 152 * 64 ? 152 * 64 : (b < 1 ? 1 : b));
}

nr_status launch_transpose(float* out, const float* in, int rows, int cols, int nviews, int M,
                           int Vs, cudaStream_t st) {
    dim3 blk(32, 8), grd(cdiv(cols, 32), cdiv(rows, 32), nviews);
    transpose_kernel<<<grd, blk, 0, st>>>(out, in, rows, cols, M, Vs);
    return launch_status();
}

}  // namespace nr

using namespace nr;

NR_API nr_status nr_compute_yry(float* yry, const float* prj, const float* scat, int64_t n,
                                void* stream) {
    if (!yry || !prj || n < 0) return NR_ERR_BAD_ARGUMENT;
    if (n == 0) return NR_OK;
    yry_kernel<<<ew_blocks(n), 256, 0, as_stream(stream)>>>(yry, prj, scat, n);
    return launch_status();
}

NR_API nr_status nr_sart_prj_diff(float* diff, const float* prj, const float* prj_est,
                                  const float* normprj, int64_t n, void* stream) {
    if (!diff || !prj || !prj_est || !normprj || n < 0) return NR_ERR_BAD_ARGUMENT;
    if (n == 0) return NR_OK;
    prj_diff_kernel<<<ew_blocks(n), 256, 0, as_stream(stream)>>>(diff, prj, prj_est, normprj, n);
    return launch_status();
}

NR_API nr_status nr_sart_line_integrals(float* line, const float* prj, const float* blank,
                                        const float* scat, int64_t n, void* stream) {
    if (!line || !prj || !blank || n < 0) return NR_ERR_BAD_ARGUMENT;
    if (n == 0) return NR_OK;
    line_kernel<<<ew_blocks(n), 256, 0, as_stream(stream)>>>(line, prj, blank, scat, n);
    return launch_status();
}

NR_API nr_status nr_compute_gamma_yry(float* out, const float* yry, const float* gamma, int64_t n,
                                      void* stream) {
    if (!out || !yry || !gamma || n < 0) return NR_ERR_BAD_ARGUMENT;
    if (n == 0) return NR_OK;
    mul_kernel<<<ew_blocks(n), 256, 0, as_stream(stream)>>>(out, yry, gamma, n);
    return launch_status();
}

NR_API nr_status nr_compute_h(float* h, const float* prj, const float* blank, const float* line,
                              const float* scat, int64_t n, void* stream) {
    if (!h || !prj || !blank || !line || n < 0) return NR_ERR_BAD_ARGUMENT;
    if (n == 0) return NR_OK;
    h_kernel<<<ew_blocks(n), 256, 0, as_stream(stream)>>>(h, prj, blank, line, scat, n);
    return launch_status();
}

NR_API nr_status nr_update_est(float* est, const float* capL, const float* RD, const float* d,
                               const float* RDD, float beta, int64_t n, void* stream) {
    if (!est || !capL || !RD || !d || !RDD || n < 0) return NR_ERR_BAD_ARGUMENT;
    if (n == 0) return NR_OK;
    update_est_kernel<<<ew_blocks(n), 256, 0, as_stream(stream)>>>(est, capL, RD, d, RDD, beta, n);
    return launch_status();
}

NR_API nr_status nr_scale(float* buf, float s, int64_t n, void* stream) {
    if (!buf || n < 0) return NR_ERR_BAD_ARGUMENT;
    if (n == 0) return NR_OK;
    scale_kernel<<<ew_blocks(n), 256, 0, as_stream(stream)>>>(buf, s, n);
    return launch_status();
}

NR_API nr_status nr_regroup(float* out, const float* in, int32_t n_angles, int32_t subset_num,
                            int64_t b_size, void* stream) {
    if (!out || !in || out == in || n_angles <= 0 || b_size <= 0) return NR_ERR_BAD_ARGUMENT;
    if (subset_num <= 0 || n_angles % subset_num != 0) return NR_ERR_BAD_GEOMETRY;
    const int Vs = n_angles / subset_num;
    int64_t bx = (b_size + 255) / 256;
    dim3 grd((unsigned)(bx > 4096 ? 4096 : bx), n_angles);
    regroup_kernel<<<grd, 256, 0, as_stream(stream)>>>(out, in, subset_num, Vs, b_size);
    return launch_status();
}

NR_API nr_status nr_x_y_flip(float* out, const float* in, int32_t nbx, int32_t nby,
                             int32_t n_views, void* stream) {
    if (!out || !in || out == in || nbx <= 0 || nby <= 0 || n_views < 0) return NR_ERR_BAD_ARGUMENT;
    if (n_views == 0) return NR_OK;
    // in[v][j][i] (rows = nby, cols = nbx) -> out[v][i][j]
    return launch_transpose(out, in, nby, nbx, n_views, 0, 1, as_stream(stream));
}
