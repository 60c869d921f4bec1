// ostr_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's OSTR path (PranjalSahu/newrecon), used as
// the parity oracle (double) and as the timed CPU baseline (float).  Only the
// tests, __graft_entry__.smoke() and bench.py's CPU legs may load this library;
// the product path never does.
//
// Parity pin: tests/golden/ holds outputs of the reference's own code
// (Tomo_OSTR.cu kernel bodies + Tomo_OSTR_gold.cpp host driver, compiled for
// the CPU by oracle/build_ref.sh) on seeded inputs; the float instantiation of
// this file is checked against those fixtures.
//
// Every routine cites the reference lines whose control flow it restates.
// Arithmetic follows the reference's operation order, including where the
// reference mixes in double literals (e.g. (i+0.5)*Bsize_x is evaluated in
// double and rounded to float), so that the float instantiation tracks the
// reference bit-closely and the double instantiation is its FP64 oracle.
//
// Build: g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC (see oracle/build.py).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/nrgb300.h"

namespace {

template <class R> struct RT;
template <> struct RT<float> {
    static float sqrt_(float v) { return std::sqrt(v); }
    static float floor_(float v) { return std::floor(v); }
    static float sin_(float v) { return std::sin(v); }
    static float cos_(float v) { return std::cos(v); }
    static float exp_(float v) { return std::exp(v); }
};
template <> struct RT<double> {
    static double sqrt_(double v) { return std::sqrt(v); }
    static double floor_(double v) { return std::floor(v); }
    static double sin_(double v) { return std::sin(v); }
    static double cos_(double v) { return std::cos(v); }
    static double exp_(double v) { return std::exp(v); }
};

// Siddon ray trace from (x0,y0,z0) to (x1,y1,z1) through the voxel grid.
// Restates rayTrace3D_GPU_direct_notexturememory_OSTR, Tomo_OSTR.cu:612-890
// (mode 0: weighted sum of the volume) and
// rayTrace3D_GPU_direct_notexturememory_normprj, Tomo_OSTR.cu:892-1173
// (mode 1: sum of in-volume chord lengths; mode 2: returns Length, :1172).
// Returns false for rays that miss the volume (status -1 in the reference).
template <class R>
bool ray_trace(const nr_geom& g, const R* vol, R x0, R y0, R z0, R x1, R y1, R z1,
               int mode, R* out) {
    typedef RT<R> M;
    const R Vx = (R)g.vx, Vy = (R)g.vy, Vz = (R)g.vz;
    const R xp0 = (R)g.x_p0, yp0 = (R)g.y_p0, zp0 = (R)g.z_p0;
    const int NX = g.nx, NY = g.ny, NZ = g.nz;
    R min_lx, max_lx, min_ly, max_ly, min_lz, max_lz, min_l, max_l, min_l_new, s_temp;
    int prev_x, prev_y, prev_z;
    R sum = 0;
    R dx = x1 - x0, dy = y1 - y0, dz = z1 - z0;
    R Length = M::sqrt_(dx * dx + dy * dy + dz * dz);

    if (x1 != x0) {                                     // :641-663
        min_lx = (xp0 - x0) / dx;
        max_lx = min_lx + (R)NX * Vx / dx;
        if (min_lx > max_lx) { s_temp = min_lx; min_lx = max_lx; max_lx = s_temp; }
    } else {
        if (x0 >= (R)NX * Vx + xp0 || x0 <= xp0) return false;
        min_lx = (R)-1e3; max_lx = (R)1e3;
    }
    if (y0 != y1) {                                     // :666-689
        min_ly = (yp0 - y0) / dy;
        max_ly = min_ly + (R)NY * Vy / dy;
        if (min_ly > max_ly) { s_temp = min_ly; min_ly = max_ly; max_ly = s_temp; }
    } else {
        if (y0 >= (R)NY * Vy + yp0 || y0 <= yp0) return false;
        min_ly = (R)-1e3; max_ly = (R)1e3;
    }
    if (z0 != z1) {                                     // :691-714
        min_lz = (zp0 - z0) / dz;
        max_lz = min_lz + (R)NZ * Vz / dz;
        if (min_lz > max_lz) { s_temp = min_lz; min_lz = max_lz; max_lz = s_temp; }
    } else {
        if (z0 >= (R)NZ * Vz + zp0 || z0 <= zp0) return false;
        min_lz = (R)-1e3; max_lz = (R)1e3;
    }
    max_l = max_lx;                                     // :716-721
    if (max_l > max_ly) max_l = max_ly;
    if (max_l > max_lz) max_l = max_lz;
    min_l = min_lx;
    if (min_l < min_ly) min_l = min_ly;
    if (min_l < min_lz) min_l = min_lz;
    if (min_l >= max_l) return false;                   // :723-726

    // First crossing per axis (:729-803).  The reference truncates the floor
    // to short; indices here stay far below 32768 so int is equivalent.
    if (min_lx != min_l) {
        prev_x = (int)(short)M::floor_((min_l * dx + x0 - xp0) / Vx);
        if (x0 < x1) min_lx = ((R)(prev_x + 1) * Vx + xp0 - x0) / dx;
        else if (x0 == x1) min_lx = (R)1e3;
        else min_lx = ((R)prev_x * Vx + xp0 - x0) / dx;
    } else {
        if (x0 < x1) { prev_x = 0; min_lx = (Vx + xp0 - x0) / dx; }
        else { prev_x = NX - 1; min_lx = ((R)prev_x * Vx + xp0 - x0) / dx; }
    }
    if (min_ly != min_l) {
        prev_y = (int)(short)M::floor_((min_l * dy + y0 - yp0) / Vy);
        if (y0 < y1) min_ly = ((R)(prev_y + 1) * Vy + yp0 - y0) / dy;
        else if (y0 == y1) min_ly = (R)1e3;
        else min_ly = ((R)prev_y * Vy + yp0 - y0) / dy;
    } else {
        if (y0 < y1) { prev_y = 0; min_ly = (Vy + yp0 - y0) / dy; }
        else { prev_y = NY - 1; min_ly = ((R)prev_y * Vy + yp0 - y0) / dy; }
    }
    if (min_lz != min_l) {
        prev_z = (int)(short)M::floor_((min_l * dz + z0 - zp0) / Vz);
        if (z0 < z1) min_lz = ((R)(prev_z + 1) * Vz + zp0 - z0) / dz;
        else if (z0 == z1) min_lz = (R)1e3;
        else min_lz = ((R)prev_z * Vz + zp0 - z0) / dz;
    } else {
        if (z0 < z1) { prev_z = 0; min_lz = (Vz + zp0 - z0) / dz; }
        else { prev_z = NZ - 1; min_lz = ((R)prev_z * Vz + zp0 - z0) / dz; }
    }

    min_l_new = min_lx;                                 // :807-809
    if (min_l_new > min_ly) min_l_new = min_ly;
    if (min_l_new > min_lz) min_l_new = min_lz;
    const R incx = Vx / dx, incy = Vy / dy, incz = Vz / dz;

    auto inside = [&]() {
        return prev_x >= 0 && prev_x < NX && prev_y >= 0 && prev_y < NY &&
               prev_z >= 0 && prev_z < NZ;
    };
    // Relative stop criterion and tie stepping exactly as :815-881.
    while ((double)((max_l - min_l_new) / max_l) > 0.000001) {
        R tmp_length = (min_l_new - min_l) * Length;
        if (inside()) {
            if (mode == 0)
                sum = sum + vol[((size_t)prev_z * NY + prev_y) * NX + prev_x] * tmp_length;
            else
                sum = sum + tmp_length;
        }
        if (min_l_new == min_lx) {
            if (x0 < x1) { prev_x += 1; min_lx = min_lx + incx; }
            else { prev_x -= 1; min_lx = min_lx - incx; }
        }
        if (min_l_new == min_ly) {
            if (y0 < y1) { prev_y += 1; min_ly = min_ly + incy; }
            else { prev_y -= 1; min_ly = min_ly - incy; }
        }
        if (min_l_new == min_lz) {
            if (z0 < z1) { prev_z += 1; min_lz = min_lz + incz; }
            else { prev_z -= 1; min_lz = min_lz - incz; }
        }
        min_l = min_l_new;
        min_l_new = min_lx;
        if (min_l_new > min_ly) min_l_new = min_ly;
        if (min_l_new > min_lz) min_l_new = min_lz;
    }
    R tmp_length = (max_l - min_l) * Length;            // :883-887
    if (inside()) {
        if (mode == 0)
            sum = sum + vol[((size_t)prev_z * NY + prev_y) * NX + prev_x] * tmp_length;
        else
            sum = sum + tmp_length;
    }
    *out = (mode == 2) ? Length : sum;
    return true;
}

// Source position and bin centre for view angle theta and bin (i, j).
// (i+0.5)*Bsize is evaluated in double, as in the reference, Tomo_OSTR.cu:1349-1350.
template <class R>
inline void bin_center(const nr_geom& g, int i, int j, R* x1, R* y1, R* z1) {
    *x1 = (R)((double)g.x_d0 + (i + 0.5) * (double)g.bx);
    *y1 = (R)((double)g.y_d0 + (j + 0.5) * (double)g.by);
    *z1 = -(R)g.detectorR;
}

// Forward projection x cos(theta) over views a in [a0,a1).
// Restates ray_trace_gpu_manyangles_direct_notexturememory_OSTR_cos,
// Tomo_OSTR.cu:1313-1376 (mode 0) and the normprj kernel :1378-1449 (modes 1, 2,
// which are NOT multiplied by cos).
template <class R>
void fp_views(const nr_geom& g, const R* vol, R* prj, const float* angles,
              const int32_t* index, int a0, int a1, int mode) {
    typedef RT<R> M;
    const int NBX = g.nbx, NBY = g.nby;
    for (int a = a0; a < a1; a++) {
        const int s = index[a];
        const R theta = (R)angles[s];
        const R st = M::sin_(theta), ct = M::cos_(theta);
        const R x0 = (R)g.sourceR * st, z0 = (R)g.sourceR * ct, y0 = (R)g.sourceY;
        R* out = prj + (size_t)(a - a0) * NBX * NBY;
#pragma omp parallel for schedule(dynamic, 4)
        for (int i = 0; i < NBX; i++) {
            for (int j = 0; j < NBY; j++) {
                R x1, y1, z1, sum;
                bin_center<R>(g, i, j, &x1, &y1, &z1);
                if (ray_trace<R>(g, vol, x0, y0, z0, x1, y1, z1, mode, &sum))
                    out[(size_t)i * NBY + j] = (mode == 0) ? sum * ct : sum;
            }
        }
    }
}

// One view's depth-weighted bilinear back projection term for voxel centre
// (x1,y1,z1) from source (x0,y0,z0), reading the [i][j] view p.  Restates the
// per-view body of backprj_gpu_manyviews_SBP, Tomo_OSTR.cu:1553-1734 (tap
// edge rules :1684-1715, depth weight :1634, Vsize_z*depth_weight scaling
// :1718); *sens gets the same interpolation of a detector of ones, the
// sensitivity of backprj_OSSART_gpu_manyviews (Tomo_OSTR.cu:1838-1882).
// Returns false (and contributes nothing) when z1 == z0.
template <class R>
inline bool bp_term(const nr_geom& g, R x0, R y0, R z0, R x1, R y1, R z1, const R* p,
                    R* u_out, R* sens_out) {
    typedef RT<R> M;
    const int NBX = g.nbx, NBY = g.nby;
    const R detR = (R)g.detectorR;
    const R depth_weight = (x0 * x0 + y0 * y0 + z0 * z0) /
        ((x0 - x1) * (x0 - x1) + (y0 - y1) * (y0 - y1) + (z0 - z1) * (z0 - z1));
    if (z1 == z0) return false;
    const R t = (-detR - z0) / (z1 - z0);
    const R x2 = x0 + (x1 - x0) * t;
    const R y2 = y0 + (y1 - y0) * t;
    const R imb = (x2 - (R)g.x_d0) / (R)g.bx;
    const R jmb = (y2 - (R)g.y_d0) / (R)g.by;
    int ilb = (int)M::floor_(imb);
    if ((double)imb < ilb + 0.5) ilb = ilb - 1;
    int jlb = (int)M::floor_(jmb);
    if ((double)jmb < jlb + 0.5) jlb = jlb - 1;
    const R fracI = (R)((double)imb - (ilb + 0.5));
    const R fracJ = (R)((double)jmb - (jlb + 0.5));
    R d1 = 0, d2 = 0, s1 = 0, s2 = 0;
    if (ilb < NBX && ilb >= 0 && jlb < NBY && jlb >= 0) {
        d1 = (1 - fracI) * p[(size_t)ilb * NBY + jlb];
        s1 = (1 - fracI);
    }
    if (ilb < NBX - 1 && ilb >= -1 && jlb < NBY && jlb >= 0) {
        d1 = d1 + fracI * p[(size_t)(ilb + 1) * NBY + jlb];
        s1 = s1 + fracI;
    }
    if (ilb < NBX && ilb >= 0 && jlb < NBY - 1 && jlb >= -1) {
        d2 = (1 - fracI) * p[(size_t)ilb * NBY + jlb + 1];
        s2 = (1 - fracI);
    }
    if (ilb < NBX - 1 && ilb >= -1 && jlb < NBY - 1 && jlb >= -1) {
        d2 = d2 + fracI * p[(size_t)(ilb + 1) * NBY + jlb + 1];
        s2 = s2 + fracI;
    }
    R u_term = (1 - fracJ) * d1 + fracJ * d2;
    *u_out = u_term * (R)g.vz * depth_weight;
    if (sens_out) {
        R u_sens = (1 - fracJ) * s1 + fracJ * s2;
        *sens_out = u_sens * (R)g.vz * depth_weight;
    }
    return true;
}

// Source of view angle theta and voxel centre (ix, iy, iz), as the back
// projectors form them (Tomo_OSTR.cu:1613-1626).
template <class R>
inline void bp_geometry(const nr_geom& g, float theta_f, int ix, int iy, int iz, R* x0, R* y0,
                        R* z0, R* x1, R* y1, R* z1) {
    typedef RT<R> M;
    const R theta = (R)theta_f;
    const R st = M::sin_(theta), ct = M::cos_(theta);
    *x0 = (R)g.sourceR * st;
    *z0 = (R)g.sourceR * ct;
    *y0 = (R)g.sourceY;
    *x1 = (R)((ix + 0.5) * (double)g.vx + (double)g.x_p0);
    *y1 = (R)((iy + 0.5) * (double)g.vy + (double)g.y_p0);
    *z1 = (R)((iz + 0.5) * (double)g.vz + (double)g.z_p0);
}

// Voxel-driven bilinear back projection, accumulated into vol
// (backprj_gpu_manyviews_SBP, Tomo_OSTR.cu:1553-1734).
template <class R>
void bp_sbp(const nr_geom& g, R* vol, const R* prj, const int32_t* index,
            const float* angles, int a0, int a1) {
    const int NX = g.nx, NY = g.ny, NZ = g.nz;
    const size_t B = (size_t)g.nbx * g.nby;
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < NZ; iz++) {
        for (int iy = 0; iy < NY; iy++) {
            for (int ix = 0; ix < NX; ix++) {
                R total_sum = 0;
                for (int a = a0; a < a1; a++) {
                    R x0, y0, z0, x1, y1, z1, u;
                    bp_geometry<R>(g, angles[index[a]], ix, iy, iz, &x0, &y0, &z0, &x1, &y1, &z1);
                    if (bp_term<R>(g, x0, y0, z0, x1, y1, z1, prj + (size_t)(a - a0) * B, &u,
                                   nullptr))
                        total_sum = total_sum + u;
                }
                size_t v = ((size_t)iz * NY + iy) * NX + ix;
                vol[v] = vol[v] + total_sum;
            }
        }
    }
}

// OS-SART update in place: x += lambda (u/s + beta prior/s), both 0 where
// s = 0, then clamp at 0.  prior == nullptr restates
// backprj_OSSART_gpu_manyviews (Tomo_OSTR.cu:1737-1936), otherwise
// backprj_OSSART_R_gpu_manyviews (:1938-2143).
template <class R>
void bp_ossart(const nr_geom& g, R* vol, const R* prj, const R* prior, const int32_t* index,
               const float* angles, int a0, int a1, R lambda, R beta) {
    const int NX = g.nx, NY = g.ny, NZ = g.nz;
    const size_t B = (size_t)g.nbx * g.nby;
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < NZ; iz++) {
        for (int iy = 0; iy < NY; iy++) {
            for (int ix = 0; ix < NX; ix++) {
                R total_sum = 0, total_sens = 0;
                for (int a = a0; a < a1; a++) {
                    R x0, y0, z0, x1, y1, z1, u, sn;
                    bp_geometry<R>(g, angles[index[a]], ix, iy, iz, &x0, &y0, &z0, &x1, &y1, &z1);
                    if (bp_term<R>(g, x0, y0, z0, x1, y1, z1, prj + (size_t)(a - a0) * B, &u,
                                   &sn)) {
                        total_sum = total_sum + u;
                        total_sens = total_sens + sn;
                    }
                }
                const size_t v = ((size_t)iz * NY + iy) * NX + ix;
                R u_term = 0, beta_term = 0;
                if (total_sens != 0) {
                    u_term = total_sum / total_sens;
                    if (prior) beta_term = (beta * prior[v]) / total_sens;
                }
                R nv = vol[v] + lambda * (u_term + beta_term);
                vol[v] = nv < 0 ? (R)0 : nv;
            }
        }
    }
}

// SART projector: est = line integral (times cos theta with use_cos), norm =
// in-volume chord (the sum_norm of the same walk), missed rays untouched.
// Restates ray_trace_gpu_manyangles_direct_notexturememory{,_cos},
// Tomo_OSTR.cu:1177-1311, with rayTrace3D_GPU_direct_notexturememory
// (:327-610), whose sum and sum_norm are the mode 0 and mode 1 walks above.
template <class R>
void fp_sart(const nr_geom& g, const R* vol, R* est, R* norm, const float* angles,
             const int32_t* index, int a0, int a1, int use_cos) {
    typedef RT<R> M;
    const int NBX = g.nbx, NBY = g.nby;
    for (int a = a0; a < a1; a++) {
        const R theta = (R)angles[index[a]];
        const R st = M::sin_(theta), ct = M::cos_(theta);
        const R x0 = (R)g.sourceR * st, z0 = (R)g.sourceR * ct, y0 = (R)g.sourceY;
        const size_t o0 = (size_t)(a - a0) * NBX * NBY;
#pragma omp parallel for schedule(dynamic, 4)
        for (int i = 0; i < NBX; i++) {
            for (int j = 0; j < NBY; j++) {
                R x1, y1, z1, sum, sn;
                bin_center<R>(g, i, j, &x1, &y1, &z1);
                if (ray_trace<R>(g, vol, x0, y0, z0, x1, y1, z1, 0, &sum)) {
                    ray_trace<R>(g, vol, x0, y0, z0, x1, y1, z1, 1, &sn);
                    est[o0 + (size_t)i * NBY + j] = use_cos ? sum * ct : sum;
                    norm[o0 + (size_t)i * NBY + j] = sn;
                }
            }
        }
    }
}

// 2 x 2 super-sampled projection, the fixed fprojectCB1_4R_GPU_SART: the
// sub-ray kernel ray_trace_4R_gpu_manyangles_direct_notexturememory
// (Tomo_OSTR.cu:1453-1515: sub-bin centre x_d0 + (i+0.5)/2*Bsize_x in double,
// plain line integral, sub layout [view][2 BINSy][2 BINSx], missed untouched)
// and the merge merge_4R_to_1R_global (:1517-1550) as intended: the four
// sub-rays (2i,2j), (2i+1,2j), (2i,2j+1), (2i+1,2j+1) summed in that order,
// / 4, with missed sub-rays 0 (a zeroed sub-ray buffer).  The merged value is
// multiplied by cos theta with use_cos; layout 0 writes [view][i][j], 1
// [view][j][i] (the merge's).
template <class R>
void fp_4r(const nr_geom& g, const R* vol, R* prj, R* sub, const float* angles,
           const int32_t* index, int a0, int a1, int use_cos, int layout) {
    typedef RT<R> M;
    const int NBX = g.nbx, NBY = g.nby, NBX2 = 2 * NBX, NBY2 = 2 * NBY;
    std::vector<R> s4((size_t)NBX2 * NBY2);
    for (int a = a0; a < a1; a++) {
        const R theta = (R)angles[index[a]];
        const R st = M::sin_(theta), ct = M::cos_(theta);
        const R x0 = (R)g.sourceR * st, z0 = (R)g.sourceR * ct, y0 = (R)g.sourceY;
#pragma omp parallel for schedule(dynamic, 4)
        for (int js = 0; js < NBY2; js++)
            for (int is = 0; is < NBX2; is++) {
                const R x1 = (R)((double)g.x_d0 + (is + 0.5) / 2 * (double)g.bx);
                const R y1 = (R)((double)g.y_d0 + (js + 0.5) / 2 * (double)g.by);
                R v;
                const bool hit = ray_trace<R>(g, vol, x0, y0, z0, x1, y1, -(R)g.detectorR, 0, &v);
                s4[(size_t)js * NBX2 + is] = hit ? v : (R)0;
                if (hit && sub) sub[((size_t)(a - a0) * NBY2 + js) * NBX2 + is] = v;
            }
        for (int j = 0; j < NBY; j++)
            for (int i = 0; i < NBX; i++) {
                const R* r0 = &s4[(size_t)(2 * j) * NBX2 + 2 * i];
                const R* r1 = r0 + NBX2;
                R m = (((r0[0] + r0[1]) + r1[0]) + r1[1]) / 4;
                if (use_cos) m = m * ct;
                const size_t o = layout ? (size_t)j * NBX + i : (size_t)i * NBY + j;
                prj[(size_t)(a - a0) * NBX * NBY + o] = m;
            }
    }
}

// SART_prj_diff_kernel, Tomo_OSTR.cu:2145-2183.
template <class R>
void sart_prj_diff(R* diff, const R* prj, const R* est, const R* norm, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) diff[i] = norm[i] != 0 ? (prj[i] - est[i]) / norm[i] : (R)0;
}

// G_Huber_prior, Tomo_OSTR.cu:258-325: prior += sum over the 26 neighbours of
// (1/distance) diff / sqrt(1 + (diff/delta)^2), plain distances, centre
// distance 1 (its diff is 0), out-of-volume neighbour = the voxel itself.
// The float instantiation keeps the reference's mixed float/double rounding.
template <class R>
void prior_sart(const nr_geom& g, R* prior, const R* x, R delta) {
    const int NX = g.nx, NY = g.ny, NZ = g.nz;
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < NZ; iz++)
        for (int iy = 0; iy < NY; iy++)
            for (int ix = 0; ix < NX; ix++) {
                const size_t v = ((size_t)iz * NY + iy) * NX + ix;
                R acc = prior[v];
                for (int kz = iz - 1; kz < iz + 2; kz++)
                    for (int ky = iy - 1; ky < iy + 2; ky++)
                        for (int kx = ix - 1; kx < ix + 2; kx++) {
                            const int ddx = kx - ix, ddy = ky - iy, ddz = kz - iz;
                            R distance = std::sqrt((R)(ddx * ddx + ddy * ddy + ddz * ddz));
                            if (distance == 0) distance = 1;
                            size_t nb = v;
                            if (!(kx < 0 || ky < 0 || kz < 0 || kx > NX - 1 || ky > NY - 1 || kz > NZ - 1))
                                nb = ((size_t)kz * NY + ky) * NX + kx;
                            const R diff = x[v] - x[nb];
                            const R den = (R)std::sqrt(1.0 + (double)((diff / delta) * (diff / delta)));
                            acc = (R)((double)acc + (1.0 / (double)distance) * (double)diff / (double)den);
                        }
                prior[v] = acc;
            }
}

// log(blank / (prj - scat)) where both are positive, else 0.
template <class R>
void line_integrals(R* line, const R* prj, const R* blank, const R* scat, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        const R nu = prj[i] - (scat ? scat[i] : (R)0);
        line[i] = (nu > 0 && blank[i] > 0) ? (R)std::log((double)blank[i] / (double)nu) : (R)0;
    }
}

// Denominator of the weight as the reference stores it (a float variable
// computed partly in double): omega(t) = 1/den(t).
//   Q2 1; Lange 1+|t/delta| (Tomo_OSTR.cu:244); hyperbola sqrt(1+(t/delta)^2)
//   (Tomo_OSTR.cu:314); Huber max(1, |t|/delta) (no reference counterpart).
template <class R>
inline R prior_den(int pot, R t, R delta) {
    switch (pot) {
    case NR_POT_Q2: return (R)1;
    case NR_POT_LANGE: return (R)(1.0 + (double)std::fabs(t / delta));
    case NR_POT_HYPERBOLA: return (R)std::sqrt(1.0 + (double)((t / delta) * (t / delta)));
    default: { R a = std::fabs(t); return a <= delta ? (R)1 : a / delta; }
    }
}
inline double psi(int pot, double t, double delta) {
    double a = std::fabs(t);
    switch (pot) {
    case NR_POT_Q2: return 0.5 * t * t;
    case NR_POT_LANGE: return delta * delta * (a / delta - std::log1p(a / delta));
    case NR_POT_HYPERBOLA: {
        // d^2 (sqrt(1+u^2) - 1) in the form without cancellation for small u
        const double u2 = (t / delta) * (t / delta);
        return delta * delta * (u2 / (std::sqrt(1.0 + u2) + 1.0));
    }
    default: return a <= delta ? 0.5 * t * t : delta * a - 0.5 * delta * delta;
    }
}

// 26-neighbour penalty gradient/curvature, accumulated into RDD and RD.
// Restates G_Q2_prior / G_Fessler_prior, Tomo_OSTR.cu:118-255: neighbour
// distance sqrt(dx^2+dy^2+(dz*z_xy_ratio)^2), centre weight 0, out-of-volume
// neighbour replaced by the voxel itself (t = 0, but its weight still adds
// to RDD).  The reference forms the weight in double from float distance and
// denominator, rounds it to float and accumulates in float; the float
// instantiation keeps that.
template <class R>
void prior(const nr_geom& g, R* RDD, R* RD, const R* x, int pot, R delta, R zxy) {
    const int NX = g.nx, NY = g.ny, NZ = g.nz;
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < NZ; iz++) {
        for (int iy = 0; iy < NY; iy++) {
            for (int ix = 0; ix < NX; ix++) {
                const size_t v = ((size_t)iz * NY + iy) * NX + ix;
                R rdd = RDD[v], rd = RD[v];
                for (int kz = iz - 1; kz < iz + 2; kz++)
                    for (int ky = iy - 1; ky < iy + 2; ky++)
                        for (int kx = ix - 1; kx < ix + 2; kx++) {
                            const int ddx = kx - ix, ddy = ky - iy, ddz = kz - iz;
                            R distance = std::sqrt((R)(ddx * ddx + ddy * ddy) +
                                                   (R)(ddz * ddz) * zxy * zxy);
                            int cent = 1;
                            if (distance == 0) { distance = 1; cent = 0; }
                            size_t nb = v;
                            if (!(kx < 0 || ky < 0 || kz < 0 || kx > NX - 1 || ky > NY - 1 || kz > NZ - 1))
                                nb = ((size_t)kz * NY + ky) * NX + kx;
                            const R diff = x[v] - x[nb];
                            const R den = prior_den<R>(pot, diff, delta);
                            const R rdd_tmp = (R)(cent * (1.0 / (double)distance) / (double)den);
                            rdd = rdd + rdd_tmp;
                            rd = rd + rdd_tmp * diff;
                        }
                RDD[v] = rdd;
                RD[v] = rd;
            }
        }
    }
}

// compute_yry, Tomo_OSTR_gold.cpp:183-205.
template <class R>
void compute_yry(R* yry, const R* prj, const R* scat, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        if (prj[i] == 0) { yry[i] = 0; continue; }
        R dif = prj[i] - (scat ? scat[i] : (R)0);
        if (dif <= 0) dif = prj[i];
        yry[i] = (dif * dif) / prj[i];
    }
}

// compute_h, Tomo_OSTR_gold.cpp:245-260.
template <class R>
void compute_h(R* h, const R* prj, const R* blank, const R* line, const R* scat, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        R y_tmp = blank[i] * RT<R>::exp_(-line[i]);
        h[i] = (prj[i] / (y_tmp + (scat ? scat[i] : (R)0)) - 1) * y_tmp;
    }
}

// update_est, Tomo_OSTR_gold.cpp:265-295.
template <class R>
void update_est(R* est, const R* capL, const R* RD, const R* d, const R* RDD, R beta, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        R v = est[i] - (capL[i] + beta * RD[i]) / (d[i] + 2 * beta * RDD[i]);
        est[i] = v < 0 ? (R)0 : v;
    }
}

// regroup_prj, Tomo_OSTR_gold.cpp:220-242: out view (i*Vs + j) = in view (j*M + i).
template <class R>
void regroup(R* out, const R* in, int n_angles, int M, int64_t b) {
    const int Vs = n_angles / M;
    for (int i = 0; i < M; i++)
        for (int j = 0; j < Vs; j++)
            std::memcpy(out + (size_t)(i * Vs + j) * b, in + (size_t)(j * M + i) * b, b * sizeof(R));
}

// Subset order of views, Tomo_OSTR_gold.cpp:628-642.
void reorder_index(int32_t* idx, int n_angles, int M) {
    std::vector<int32_t> tmp(idx, idx + n_angles);
    const int Vs = n_angles / M;
    int flag = 0;
    for (int i = 0; i < M; i++)
        for (int j = 0; j < Vs; j++) idx[flag++] = tmp[j * M + i];
}

// Whole reconstruction in the order of ConebeamCT_OSTR_LangePrior_GPU /
// ConebeamCT_OSTR_Q2Prior_GPU, Tomo_OSTR_gold.cpp:301-918 / 920-1469:
// yry; gamma over all views (identity order); d = SBP(gamma*yry); regroup
// prj/scat/blank; reorder index; per iter, per subset: FP_cos -> h -> SBP ->
// x M -> prior -> update.  x holds x0 on entry and the result on exit.
template <class R>
void reconstruct(const nr_geom& g, const nr_ostr_params& p, const float* angles,
                 const R* prj_in, const R* blank_in, const R* scat_in, R* x, int iters,
                 R* d_out, R* gamma_out) {
    const int A = g.n_angles, M = p.subset_num, Vs = A / M;
    const int64_t B = (int64_t)g.nbx * g.nby, N = (int64_t)g.nx * g.ny * g.nz;
    const int64_t AB = (int64_t)A * B;
    std::vector<int32_t> index(A);
    for (int i = 0; i < A; i++) index[i] = i;
    std::vector<R> yry(AB), gamma(AB, 0), d(N, 0);
    compute_yry<R>(yry.data(), prj_in, scat_in, AB);
    fp_views<R>(g, nullptr, gamma.data(), angles, index.data(), 0, A,
                p.gamma_mode == NR_GAMMA_CHORD ? 1 : 2);
    if (gamma_out) std::copy(gamma.begin(), gamma.end(), gamma_out);
    for (int64_t i = 0; i < AB; i++) yry[i] = yry[i] * gamma[i];   // compute_gamma_yry :208-218
    bp_sbp<R>(g, d.data(), yry.data(), index.data(), angles, 0, A);
    if (d_out) std::copy(d.begin(), d.end(), d_out);
    std::vector<R> prj(AB), blank(AB), scat(scat_in ? AB : 0);
    regroup<R>(prj.data(), prj_in, A, M, B);
    regroup<R>(blank.data(), blank_in, A, M, B);
    if (scat_in) regroup<R>(scat.data(), scat_in, A, M, B);
    reorder_index(index.data(), A, M);
    const R zxy = (R)(g.vz / g.vx);
    std::vector<R> line((size_t)Vs * B), h((size_t)Vs * B), capL(N), RDD(N), RD(N);
    for (int iter = 0; iter < iters; iter++) {
        for (int a = 0; a < M; a++) {
            const int a0 = a * Vs, a1 = (a + 1) * Vs;
            std::fill(line.begin(), line.end(), (R)0);
            std::fill(capL.begin(), capL.end(), (R)0);
            std::fill(RDD.begin(), RDD.end(), (R)0);
            std::fill(RD.begin(), RD.end(), (R)0);
            fp_views<R>(g, x, line.data(), angles, index.data(), a0, a1, 0);
            compute_h<R>(h.data(), prj.data() + a0 * B, blank.data() + a0 * B, line.data(),
                         scat_in ? scat.data() + a0 * B : nullptr, (int64_t)Vs * B);
            bp_sbp<R>(g, capL.data(), h.data(), index.data(), angles, a0, a1);
            for (int64_t i = 0; i < N; i++) capL[i] = (R)M * capL[i];
            prior<R>(g, RDD.data(), RD.data(), x, p.potential, (R)p.delta, zxy);
            update_est<R>(x, capL.data(), RD.data(), d.data(), RDD.data(), (R)p.beta, N);
        }
    }
}

// One sub-iteration of the loop body of Tomo_OSTR_gold.cpp:727-856 on the
// subset views [a0, a1) of the (reordered) index; prj/blank/scat hold that
// subset's views.  Used to time the CPU path per sub-iteration.
template <class R>
void subiter(const nr_geom& g, const nr_ostr_params& p, const float* angles,
             const int32_t* index, int a0, int a1, const R* prj, const R* blank,
             const R* scat, const R* d, R* x) {
    const int64_t B = (int64_t)g.nbx * g.nby, N = (int64_t)g.nx * g.ny * g.nz;
    const int Vs = a1 - a0;
    std::vector<R> line((size_t)Vs * B, 0), h((size_t)Vs * B), capL(N, 0), RDD(N, 0), RD(N, 0);
    fp_views<R>(g, x, line.data(), angles, index, a0, a1, 0);
    compute_h<R>(h.data(), prj, blank, line.data(), scat, (int64_t)Vs * B);
    bp_sbp<R>(g, capL.data(), h.data(), index, angles, a0, a1);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) capL[i] = (R)p.subset_num * capL[i];
    prior<R>(g, RDD.data(), RD.data(), x, p.potential, (R)p.delta, (R)(g.vz / g.vx));
    update_est<R>(x, capL.data(), RD.data(), d, RDD.data(), (R)p.beta, N);
}

// Mean in-volume chord of the 2 x 2 sub-rays of each bin ([view][i][j]), merged
// in the order of fp_4r, missed sub-rays 0: the normprj of the super-sampled
// OS-SART loop.
template <class R>
void fp_4r_chord(const nr_geom& g, R* norm, const float* angles, const int32_t* index, int a0,
                 int a1) {
    typedef RT<R> M;
    const int NBX = g.nbx, NBY = g.nby;
    for (int a = a0; a < a1; a++) {
        const R theta = (R)angles[index[a]];
        const R st = M::sin_(theta), ct = M::cos_(theta);
        const R x0 = (R)g.sourceR * st, z0 = (R)g.sourceR * ct, y0 = (R)g.sourceY;
#pragma omp parallel for schedule(dynamic, 4)
        for (int i = 0; i < NBX; i++)
            for (int j = 0; j < NBY; j++) {
                R c[4];
                for (int k = 0; k < 4; k++) {
                    const int is = 2 * i + (k & 1), js = 2 * j + (k >> 1);
                    const R x1 = (R)((double)g.x_d0 + (is + 0.5) / 2 * (double)g.bx);
                    const R y1 = (R)((double)g.y_d0 + (js + 0.5) / 2 * (double)g.by);
                    R v;
                    c[k] = ray_trace<R>(g, (const R*)nullptr, x0, y0, z0, x1, y1,
                                        -(R)g.detectorR, 1, &v) ? v : (R)0;
                }
                norm[(size_t)(a - a0) * NBX * NBY + (size_t)i * NBY + j] =
                    (((c[0] + c[1]) + c[2]) + c[3]) / 4;
            }
    }
}

// The OS-SART loop of the device-resident path: line integrals ([view][i][j],
// original order) regrouped to subset order, subset-major index
// (Tomo_OSTR_gold.cpp:628-642); per iteration and subset: est, norm zeroed
// (missed rays: difference 0), fp_sart, sart_prj_diff, [prior zeroed +
// prior_sart], bp_ossart in place.
template <class R>
void ossart(const nr_geom& g, const nr_sart_params& p, const float* angles, const R* line_in,
            R* x, int iters) {
    const int A = g.n_angles, M = p.subset_num, Vs = A / M;
    const int64_t B = (int64_t)g.nbx * g.nby, N = (int64_t)g.nx * g.ny * g.nz;
    std::vector<int32_t> index(A);
    for (int i = 0; i < A; i++) index[i] = i;
    reorder_index(index.data(), A, M);
    std::vector<R> line((size_t)A * B);
    regroup<R>(line.data(), line_in, A, M, B);
    std::vector<R> est((size_t)Vs * B), norm((size_t)Vs * B), diff((size_t)Vs * B);
    std::vector<R> prior(p.regularized ? N : 0);
    for (int iter = 0; iter < iters; iter++)
        for (int a = 0; a < M; a++) {
            const int a0 = a * Vs, a1 = a0 + Vs;
            std::fill(est.begin(), est.end(), (R)0);
            std::fill(norm.begin(), norm.end(), (R)0);
            if (p.supersample) {
                // 2 x 2 sub-rays: the merged projection and the merged chord
                fp_4r<R>(g, x, est.data(), nullptr, angles, index.data(), a0, a1, p.use_cos, 0);
                fp_4r_chord<R>(g, norm.data(), angles, index.data(), a0, a1);
            } else {
                fp_sart<R>(g, x, est.data(), norm.data(), angles, index.data(), a0, a1,
                           p.use_cos);
            }
            sart_prj_diff<R>(diff.data(), line.data() + (size_t)a0 * B, est.data(), norm.data(),
                             (int64_t)Vs * B);
            if (p.regularized) {
                std::fill(prior.begin(), prior.end(), (R)0);
                prior_sart<R>(g, prior.data(), x, (R)p.delta);
            }
            bp_ossart<R>(g, x, diff.data(), p.regularized ? prior.data() : nullptr, index.data(),
                         angles, a0, a1, (R)p.lambda, (R)p.beta);
        }
}

}  // namespace

#define ORC_EXPORT extern "C" __attribute__((visibility("default")))

#define ORC_INSTANTIATE(R, SUF)                                                         \
    ORC_EXPORT void orc_fp_ostr_##SUF(const nr_geom* g, const R* x, R* line,            \
                                      const float* angles, const int32_t* index,        \
                                      int a0, int a1) {                                 \
        fp_views<R>(*g, x, line, angles, index, a0, a1, 0);                             \
    }                                                                                   \
    ORC_EXPORT void orc_fp_gamma_##SUF(const nr_geom* g, R* gamma, const float* angles, \
                                       const int32_t* index, int a0, int a1, int mode) {\
        fp_views<R>(*g, (const R*)nullptr, gamma, angles, index, a0, a1,                \
                    mode == NR_GAMMA_CHORD ? 1 : 2);                                    \
    }                                                                                   \
    ORC_EXPORT void orc_bp_sbp_##SUF(const nr_geom* g, R* vol, const R* prj,            \
                                     const int32_t* index, const float* angles,         \
                                     int a0, int a1) {                                  \
        bp_sbp<R>(*g, vol, prj, index, angles, a0, a1);                                 \
    }                                                                                   \
    ORC_EXPORT void orc_prior_##SUF(const nr_geom* g, R* RDD, R* RD, const R* x,        \
                                    int pot, double delta, double zxy) {                \
        prior<R>(*g, RDD, RD, x, pot, (R)delta, (R)zxy);                                \
    }                                                                                   \
    ORC_EXPORT void orc_compute_yry_##SUF(R* yry, const R* prj, const R* scat,          \
                                          int64_t n) {                                  \
        compute_yry<R>(yry, prj, scat, n);                                              \
    }                                                                                   \
    ORC_EXPORT void orc_compute_h_##SUF(R* h, const R* prj, const R* blank,             \
                                        const R* line, const R* scat, int64_t n) {      \
        compute_h<R>(h, prj, blank, line, scat, n);                                     \
    }                                                                                   \
    ORC_EXPORT void orc_update_est_##SUF(R* est, const R* capL, const R* RD,            \
                                         const R* d, const R* RDD, double beta,         \
                                         int64_t n) {                                   \
        update_est<R>(est, capL, RD, d, RDD, (R)beta, n);                               \
    }                                                                                   \
    ORC_EXPORT void orc_regroup_##SUF(R* out, const R* in, int n_angles, int M,         \
                                      int64_t b) {                                      \
        regroup<R>(out, in, n_angles, M, b);                                            \
    }                                                                                   \
    ORC_EXPORT void orc_subiter_##SUF(const nr_geom* g, const nr_ostr_params* p,          \
                                      const float* angles, const int32_t* index, int a0,  \
                                      int a1, const R* prj, const R* blank, const R* scat, \
                                      const R* d, R* x) {                                 \
        subiter<R>(*g, *p, angles, index, a0, a1, prj, blank, scat, d, x);                \
    }                                                                                   \
    ORC_EXPORT void orc_reconstruct_##SUF(const nr_geom* g, const nr_ostr_params* p,    \
                                          const float* angles, const R* prj,            \
                                          const R* blank, const R* scat, R* x,          \
                                          int iters, R* d_out, R* gamma_out) {          \
        reconstruct<R>(*g, *p, angles, prj, blank, scat, x, iters, d_out, gamma_out);   \
    }

#define ORC_INSTANTIATE_SART(R, SUF)                                                    \
    ORC_EXPORT void orc_fp_sart_##SUF(const nr_geom* g, const R* x, R* est, R* norm,    \
                                      const float* angles, const int32_t* index,        \
                                      int a0, int a1, int use_cos) {                    \
        fp_sart<R>(*g, x, est, norm, angles, index, a0, a1, use_cos);                   \
    }                                                                                   \
    ORC_EXPORT void orc_fp_4r_##SUF(const nr_geom* g, const R* x, R* prj, R* sub,         \
                                    const float* angles, const int32_t* index, int a0,  \
                                    int a1, int use_cos, int layout) {                  \
        fp_4r<R>(*g, x, prj, sub, angles, index, a0, a1, use_cos, layout);              \
    }                                                                                   \
    ORC_EXPORT void orc_sart_prj_diff_##SUF(R* diff, const R* prj, const R* est,        \
                                            const R* norm, int64_t n) {                 \
        sart_prj_diff<R>(diff, prj, est, norm, n);                                      \
    }                                                                                   \
    ORC_EXPORT void orc_bp_ossart_##SUF(const nr_geom* g, R* x, const R* diff,          \
                                        const R* prior, const int32_t* index,           \
                                        const float* angles, int a0, int a1,            \
                                        double lambda, double beta) {                   \
        bp_ossart<R>(*g, x, diff, prior, index, angles, a0, a1, (R)lambda, (R)beta);    \
    }                                                                                   \
    ORC_EXPORT void orc_prior_sart_##SUF(const nr_geom* g, R* prior, const R* x,        \
                                         double delta) {                                \
        prior_sart<R>(*g, prior, x, (R)delta);                                          \
    }                                                                                   \
    ORC_EXPORT void orc_line_integrals_##SUF(R* line, const R* prj, const R* blank,     \
                                             const R* scat, int64_t n) {                \
        line_integrals<R>(line, prj, blank, scat, n);                                   \
    }                                                                                   \
    ORC_EXPORT void orc_ossart_##SUF(const nr_geom* g, const nr_sart_params* p,         \
                                     const float* angles, const R* line, R* x,          \
                                     int iters) {                                       \
        ossart<R>(*g, *p, angles, line, x, iters);                                      \
    }

ORC_INSTANTIATE(float, f32)
ORC_INSTANTIATE_SART(float, f32)
ORC_INSTANTIATE_SART(double, f64)
ORC_INSTANTIATE(double, f64)

ORC_EXPORT void orc_reorder_index(int32_t* idx, int n_angles, int M) {
    reorder_index(idx, n_angles, M);
}

// FP64 penalized-likelihood objective (the reference has none; the form is the
// Poisson transmission log-likelihood with the same FP_cos forward model, and
// the 26-neighbour penalty R(x) = 1/2 sum_j sum_k w_jk psi(x_j - x_k)).
// out[0] = data term, out[1] = penalty (multiply by beta for the total).
// prj/blank/scat are in ORIGINAL view order with identity index.
ORC_EXPORT void orc_objective_f64(const nr_geom* g, const nr_ostr_params* p,
                                  const float* angles, const double* prj,
                                  const double* blank, const double* scat,
                                  const double* x, double* out) {
    const int A = g->n_angles;
    const int64_t B = (int64_t)g->nbx * g->nby;
    std::vector<int32_t> index(A);
    for (int i = 0; i < A; i++) index[i] = i;
    std::vector<double> line((size_t)A * B, 0.0);
    fp_views<double>(*g, x, line.data(), angles, index.data(), 0, A, 0);
    double data = 0;
#pragma omp parallel for reduction(+ : data) schedule(static)
    for (int64_t i = 0; i < (int64_t)A * B; i++) {
        double yb = blank[i] * std::exp(-line[i]);
        double r = scat ? scat[i] : 0.0;
        double m = yb + r;
        data += m - (prj[i] > 0 ? prj[i] * std::log(m) : 0.0);
    }
    const int NX = g->nx, NY = g->ny, NZ = g->nz;
    const double zxy = (double)g->vz / (double)g->vx;
    double pen = 0;
#pragma omp parallel for collapse(2) reduction(+ : pen) schedule(static)
    for (int iz = 0; iz < NZ; iz++)
        for (int iy = 0; iy < NY; iy++)
            for (int ix = 0; ix < NX; ix++) {
                const size_t v = ((size_t)iz * NY + iy) * NX + ix;
                for (int kz = iz - 1; kz <= iz + 1; kz++)
                    for (int ky = iy - 1; ky <= iy + 1; ky++)
                        for (int kx = ix - 1; kx <= ix + 1; kx++) {
                            if (kx == ix && ky == iy && kz == iz) continue;
                            if (kx < 0 || ky < 0 || kz < 0 || kx >= NX || ky >= NY || kz >= NZ)
                                continue;  // replaced by the voxel itself: t = 0, psi(0) = 0
                            const int ddx = kx - ix, ddy = ky - iy, ddz = kz - iz;
                            const double w = 1.0 / std::sqrt((double)(ddx * ddx + ddy * ddy) +
                                                             (double)(ddz * ddz) * zxy * zxy);
                            const size_t nb = ((size_t)kz * NY + ky) * NX + kx;
                            pen += 0.5 * w * psi(p->potential, x[v] - x[nb], (double)p->delta);
                        }
            }
    out[0] = data;
    out[1] = pen;
}

ORC_EXPORT void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

ORC_EXPORT int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
