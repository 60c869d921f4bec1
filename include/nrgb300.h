/*
 * nrgb300.h -- C ABI of the GB300 OSTR reconstruction library (libnrgb300.so).
 *
 * Ordered-subsets transmission (OSTR) penalized-likelihood reconstruction for
 * digital breast tomosynthesis.  Every entry point takes plain device pointers,
 * element counts and a CUDA stream handle (passed as void*), returns an
 * nr_status and never allocates: buffers (including scratch workspace) belong
 * to the caller.  Geometry travels by value into the kernels, so the library
 * holds no global state and calls on different streams may overlap.  The one
 * exception is nr_penalty_fp64_static, which keeps its scratch in a
 * per-device array inside the library: calls to it must not overlap.
 *
 * Layouts (the reference's, PranjalSahu/newrecon):
 *   volume       [z][y][x], x fastest            (Tomo_OSTR.cu:538, :1604)
 *   projections  [view][i<BINSx][j<BINSy], j fastest, after x_y_flip
 *                                                 (Tomo_OSTR.cu:1365,
 *                                                  Tomo_OSTR_gold.cpp:93-105)
 *   index        int32 view order; [a0, a1) is half-open and indexes the
 *                reordered index (Tomo_OSTR_gold.cpp:451)
 *
 * Every projector / back projector / prior ACCUMULATES or leaves untouched
 * exactly what the reference does, so existing callers keep their
 * zero-the-buffer-first discipline (Tomo_OSTR_gold.cpp:843-846).
 */
#ifndef NRGB300_H
#define NRGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  Replaces the reference's printf + exit(1) error paths
 * (Tomo_OSTR_gold.cpp:121-125, Tomo_OSTR.cu:2232-2236, :2627-2630). */
typedef enum nr_status {
    NR_OK = 0,
    NR_ERR_BAD_GEOMETRY = 1,   /* sizes <= 0, Vx != Vy, subset count not dividing views ... */
    NR_ERR_BAD_ARGUMENT = 2,   /* null pointer, bad view range, delta <= 0, unknown enum */
    NR_ERR_LAUNCH = 3,         /* a kernel launch failed */
    NR_ERR_NONFINITE = 4,      /* NaN/Inf detected by a device status word */
    NR_ERR_TIMEOUT = 5,        /* a bounded device wait gave up */
    NR_ERR_WORKSPACE = 6,      /* workspace missing, too small or misaligned */
    NR_ERR_CUDA = 7            /* any other CUDA runtime error */
} nr_status;

/* Scanner + grid geometry.  Field-for-field the reference's host globals
 * h_IMGSIZx ... h_sourceY (Tomo_OSTR.cu:21-36, :47-50) and ostr.py:21-52. */
typedef struct nr_geom {
    int32_t nx, ny, nz;        /* IMGSIZx, IMGSIZy, IMGSIZz (voxels)            */
    float vx, vy, vz;          /* Vsize_x, Vsize_y, Vsize_z (mm)                 */
    float x_p0, y_p0, z_p0;    /* volume corner (mm)                             */
    int32_t nbx, nby;          /* BINSx, BINSy (detector bins)                   */
    float bx, by;              /* Bsize_x, Bsize_y (mm)                          */
    float x_d0, y_d0;          /* detector corner (mm)                           */
    float detectorR;           /* detector plane at z = -detectorR (mm)          */
    float sourceR;             /* source at (R sin t, sourceY, R cos t) (mm)     */
    float sourceY;
    int32_t n_angles;          /* ANGLES                                         */
} nr_geom;

/* Penalty potentials (RDD += w*omega(t), RD += w*omega(t)*t, t = x_j - x_k). */
enum {
    NR_POT_Q2 = 0,         /* omega = 1                       G_Q2_prior      Tomo_OSTR.cu:118-184 */
    NR_POT_LANGE = 1,      /* omega = 1/(1+|t|/delta)         G_Fessler_prior Tomo_OSTR.cu:187-255 */
    NR_POT_HYPERBOLA = 2,  /* omega = 1/sqrt(1+(t/delta)^2)   formula of      Tomo_OSTR.cu:314     */
    NR_POT_HUBER = 3       /* omega = min(1, delta/|t|)       (no reference counterpart)           */
};

/* Normalisation projection gamma. */
enum {
    NR_GAMMA_LENGTH = 0,   /* full source-to-bin length |src - bin| (Tomo_OSTR.cu:1172) */
    NR_GAMMA_CHORD = 1     /* in-volume chord length (ostr.py:641, ostr.ipynb:815)      */
};

/* ---------------------------------------------------------------------------
 * Geometry check.  Replaces the reference's scattered exit(1) checks:
 * Vx == Vy (Tomo_OSTR_gold.cpp:380-386), subset_num | ANGLES
 * (Tomo_OSTR.cu:2627-2630).  subset_num <= 0 skips the subset check.
 * ------------------------------------------------------------------------- */
nr_status nr_validate_geometry(const nr_geom* g, int32_t subset_num);

/* ---------------------------------------------------------------------------
 * Reference-shaped operators (drop-in for the launch wrappers).
 * ------------------------------------------------------------------------- */

/* line[(a-a0)][i][j] = cos(theta) * Siddon line integral of x for views
 * index[a], a in [a0,a1).  Rays that miss the volume leave line untouched.
 * Replaces fprojectCB_1R_GPU_OSTR_cos (Tomo_OSTR.cu:2334-2359; kernel :1313). */
nr_status nr_fp_ostr(const nr_geom* g, const float* x, float* line,
                     const float* angles, const int32_t* index,
                     int32_t a0, int32_t a1, void* stream);

/* gamma[(a-a0)][i][j] for rays that hit the volume (others untouched).
 * mode = NR_GAMMA_LENGTH | NR_GAMMA_CHORD.
 * Replaces fprojectCB_1R_GPU_OSTR_normprj (Tomo_OSTR.cu:2361-2393; :1378). */
nr_status nr_fp_gamma(const nr_geom* g, float* gamma,
                      const float* angles, const int32_t* index,
                      int32_t a0, int32_t a1, int32_t mode, void* stream);

/* vol[j] += sum over views of the voxel-driven bilinear back projection of
 * prj (SBP, depth weighted).  Deterministic gather, no atomics.
 * Replaces bprojectCB_GPU_SBP (Tomo_OSTR.cu:2435-2457; kernel :1553). */
nr_status nr_bp_sbp(const nr_geom* g, float* vol, const float* prj,
                    const int32_t* index, const float* angles,
                    int32_t a0, int32_t a1, void* stream);

/* RDD += sum_k w_k omega(t), RD += sum_k w_k omega(t) t over the 26-neighbourhood.
 * Replaces prior_GPU_OSTR (Lange, Tomo_OSTR.cu:2216-2245) and
 * prior_GPU_OSTR_Q2 (Tomo_OSTR.cu:2189-2213).  delta must be > 0 unless Q2. */
nr_status nr_prior(const nr_geom* g, float* RDD, float* RD, const float* x,
                   int32_t potential, float delta, float z_xy_ratio, void* stream);

/* Element-wise host helpers of the reference, on the device. */
/* compute_yry (Tomo_OSTR_gold.cpp:183-205); scat may be NULL (r = 0). */
nr_status nr_compute_yry(float* yry, const float* prj, const float* scat,
                         int64_t n, void* stream);
/* compute_gamma_yry (Tomo_OSTR_gold.cpp:208-218). */
nr_status nr_compute_gamma_yry(float* out, const float* yry, const float* gamma,
                               int64_t n, void* stream);
/* compute_h (Tomo_OSTR_gold.cpp:245-260); scat may be NULL. */
nr_status nr_compute_h(float* h, const float* prj, const float* blank,
                       const float* line, const float* scat, int64_t n, void* stream);
/* update_est (Tomo_OSTR_gold.cpp:265-295), in place on est. */
nr_status nr_update_est(float* est, const float* capL, const float* RD,
                        const float* d, const float* RDD, float beta,
                        int64_t n, void* stream);
/* buf *= s (the x subset_num scaling of capL, Tomo_OSTR_gold.cpp:767-771). */
nr_status nr_scale(float* buf, float s, int64_t n, void* stream);
/* regroup_prj (Tomo_OSTR_gold.cpp:220-242): out view (i*Vs + j) = in view (j*M + i). */
nr_status nr_regroup(float* out, const float* in, int32_t n_angles,
                     int32_t subset_num, int64_t b_size, void* stream);
/* x_y_flip (Tomo_OSTR_gold.cpp:93-105) for n_views views: out[v][i][j] = in[v][j][i]. */
nr_status nr_x_y_flip(float* out, const float* in, int32_t nbx, int32_t nby,
                      int32_t n_views, void* stream);

/* ---------------------------------------------------------------------------
 * Fused device-resident OSTR (no reference counterpart as one call: it is the
 * whole loop of ConebeamCT_OSTR_{LangePrior,Q2Prior}_GPU,
 * Tomo_OSTR_gold.cpp:301-918 / :920-1469, kept on the GPU).
 * ------------------------------------------------------------------------- */
typedef struct nr_ostr_params {
    int32_t subset_num;        /* M; must divide n_angles                        */
    int32_t potential;         /* NR_POT_*                                       */
    int32_t gamma_mode;        /* NR_GAMMA_*                                     */
    int32_t has_scatter;       /* 0: r = 0 everywhere                            */
    float beta;                /* penalty weight                                 */
    float delta;               /* potential scale (1/mm), > 0 unless Q2          */
    int32_t fp_batch;          /* Siddon steps per gather round: 2, 4, 8 (0 = 4) */
    int32_t upd_planes;        /* z planes per update block: 8, 16, 32 (0 = 16) */
    int32_t fp_stage;          /* NR_STAGE_OFF (default): the projection gathers
                                  the volume through L1/L2; NR_STAGE_TMA: it stages
                                  the volume slab by slab in shared memory by TMA
                                  where the volume allows it (IMGSIZx a multiple of
                                  4, x 16-byte aligned; fp_batch 2 or 4).  Same
                                  result either way; on the clinical workload the
                                  staged form is slower (0.255 vs 0.162 ms).     */
    int32_t upd_tile;          /* NR_TILE_1 (default): the update gives each thread
                                  one voxel of a 32 x 8-column tile; NR_TILE_2: two
                                  voxels side by side in x of a 64 x 8-column tile
                                  (one-view subsets; others use NR_TILE_1).  Same
                                  result bit for bit; fewer instructions per voxel,
                                  fewer resident blocks.  NR_TILE_TMA: the
                                  one-voxel tile with its planes streamed by TMA
                                  through a shared-memory ring by a producer warp
                                  (IMGSIZx a multiple of 4 and x 16-byte aligned,
                                  else NR_TILE_1); same result bit for bit.       */
} nr_ostr_params;

enum {
    NR_STAGE_OFF = 0,
    NR_STAGE_TMA = 1
};

enum {
    NR_TILE_1 = 0,
    NR_TILE_2 = 1,
    NR_TILE_TMA = 2
};

/* fp_batch, fp_stage, upd_planes and upd_tile select kernel variants only
 * (every variant gives the same result); the autotuner
 * (newrecon_gb300/autotune.py) picks them per geometry.  The batched path
 * uses the defaults. */

/* Bytes of workspace the fused path needs for this geometry and parameters. */
nr_status nr_ostr_workspace_size(const nr_geom* g, const nr_ostr_params* p,
                                 size_t* bytes);

/* Load the scan into the workspace and precompute the curvature d.
 * prj, blank, scat: [view][i][j] in ORIGINAL view order (scat may be NULL).
 * angles: n_angles float32 radians (device).  Equivalent to lines
 * Tomo_OSTR_gold.cpp:409-642 (yry, gamma, gamma*yry, d, regroup, reorder). */
nr_status nr_ostr_setup(const nr_geom* g, const nr_ostr_params* p,
                        const float* angles, const float* prj, const float* blank,
                        const float* scat, void* workspace, size_t ws_bytes,
                        void* stream);

/* First half of sub-iteration `subset`: the fused forward projection of x
 * over the subset's views and the OSTR detector gradient
 * h = (y/(b e^-l + r) - 1) b e^-l into the workspace (Tomo_OSTR_gold.cpp:732-756). */
nr_status nr_ostr_project(const nr_geom* g, const nr_ostr_params* p, const float* x,
                          int32_t subset, void* workspace, size_t ws_bytes, void* stream);

/* Second half: x_out = max(0, x - (M SBP(h) + beta RD)/(d + 2 beta RDD)) with
 * the penalty of x, fused (Tomo_OSTR_gold.cpp:759-814).  x_out != x. */
nr_status nr_ostr_update(const nr_geom* g, const nr_ostr_params* p, const float* x,
                         float* x_out, int32_t subset, void* workspace, size_t ws_bytes,
                         void* stream);

/* Workspace sections a caller may read (device pointer + byte size). */
enum {
    NR_WS_D = 0,          /* float[N]: curvature d                                   */
    NR_WS_H = 1,          /* float[Vs][BINSy][BINSx]: last subset gradient h         */
    NR_WS_Y = 2,          /* float[A][BINSy][BINSx]: counts, subset order            */
    NR_WS_GAMMA_YRY = 3,  /* float[A][BINSy][BINSx]: gamma*yry, original order       */
    NR_WS_INDEX = 4       /* int32[A]: subset-major view order                       */
};
nr_status nr_ostr_workspace_section(const nr_geom* g, const nr_ostr_params* p,
                                    int32_t section, void* workspace, size_t ws_bytes,
                                    void** ptr, size_t* bytes);

/* Run n_iters full iterations (M sub-iterations each) on x in place
 * ([z][y][x], non-negative).  Equivalent to Tomo_OSTR_gold.cpp:724-887. */
nr_status nr_ostr_iterate(const nr_geom* g, const nr_ostr_params* p, float* x,
                          int32_t n_iters, void* workspace, size_t ws_bytes,
                          void* stream);

/* One sub-iteration for subset a (0 <= a < M), x in place. */
nr_status nr_ostr_subiter(const nr_geom* g, const nr_ostr_params* p, float* x,
                          int32_t subset, void* workspace, size_t ws_bytes,
                          void* stream);

/* Captures n_iters iterations of nr_ostr_iterate on x (fixed pointers: x and
 * the workspace are baked in) into a CUDA graph and instantiates it; *graph
 * receives an opaque handle.  stream must be a non-default stream (capture
 * runs on it; nothing executes).  The handle is host memory owned by the
 * caller: release it with nr_ostr_graph_destroy.  No reference counterpart
 * (the reference relaunches and synchronises every kernel). */
nr_status nr_ostr_graph_create(const nr_geom* g, const nr_ostr_params* p, float* x,
                               int32_t n_iters, void* workspace, size_t ws_bytes,
                               void* stream, void** graph);
/* Replays a captured graph (iteration loop or batch) on stream. */
nr_status nr_ostr_graph_launch(void* graph, void* stream);
/* Releases a graph handle (NULL is a no-op). */
nr_status nr_ostr_graph_destroy(void* graph);

/* ---------------------------------------------------------------------------
 * Batched reconstructions (no reference counterpart: the reference runs one
 * case per process).  Each case has its own geometry, parameters, volume and
 * workspace (set up with nr_ostr_setup); a batch step advances every
 * unfinished case by one sub-iteration with one projection launch and one
 * update launch per (potential, one-view, slab depth) class over all cases'
 * work items, one block per item.  Up to 64 cases.
 * ------------------------------------------------------------------------- */
typedef struct nr_batch_case {
    nr_geom g;
    nr_ostr_params p;
    int32_t n_iters;       /* iterations of this case (n_iters * M sub-iterations) */
    float* x;              /* volume, updated in place                            */
    void* workspace;       /* this case's workspace after nr_ostr_setup           */
    size_t ws_bytes;
} nr_batch_case;

/* Bytes of the case table describing n_cases cases (host memory: every batch
 * launch takes the table as its kernel parameter). */
nr_status nr_batch_table_size(int32_t n_cases, size_t* bytes);
/* Writes the case table (8-byte aligned HOST memory of nr_batch_table_size
 * bytes) and returns the number of batch steps (the largest n_iters * M).
 * Issues no GPU work (stream is not used). */
nr_status nr_batch_prepare(const nr_batch_case* cases, int32_t n_cases, void* table,
                           size_t table_bytes, int32_t* n_steps, void* stream);
/* One batch step (step = 0, 1, ... in order).  The table is read when the
 * call is made: it may be changed or freed once the call returns. */
nr_status nr_batch_step(const void* table, int32_t step, void* stream);
/* After the last step: moves results that ended in the ping-pong buffer into x. */
nr_status nr_batch_finish(const void* table, void* stream);
/* Captures steps 0 .. n_steps-1 and the finish into a CUDA graph (replay with
 * nr_ostr_graph_launch, release with nr_ostr_graph_destroy); stream must be a
 * non-default stream.  The graph keeps the table as it was at capture. */
nr_status nr_batch_graph_create(const void* table, int32_t n_steps, void* stream, void** graph);

/* ---------------------------------------------------------------------------
 * Learned warm start (no reference counterpart; the nearest is the Keras 3D
 * U-Net post-processor of recon1.ipynb:211).  A 3D residual CNN of six
 * 3x3x3 convolutions (1 -> 32 -> 32 -> 32 -> 32 -> 32 -> 1 channels, ReLU)
 * maps an early OSTR iterate x to x_warm = max(0, x + f(s x) / s), with BF16
 * weights and activations on the tensor cores and FP32 accumulation.  Volumes
 * are nb patches of nx x ny x nz voxels stored back to back ([b][z][y][x]);
 * each patch is zero-padded at its own borders.  Parameters are one FP32
 * array: for each layer W[27][out][in] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1))
 * then b[out].
 * ------------------------------------------------------------------------- */
typedef struct nr_cnn_dims {
    int32_t nx, ny, nz, nb;
} nr_cnn_dims;

/* Number of FP32 parameters. */
nr_status nr_cnn_param_count(int64_t* n);
/* Workspace bytes for inference (training = 0) or training (training = 1). */
nr_status nr_cnn_workspace_size(const nr_cnn_dims* d, int32_t training, size_t* bytes);
/* x_out = max(0, x + f(s x)/s); s = in_scale > 0. */
nr_status nr_cnn_forward(const nr_cnn_dims* d, const float* params, const float* x,
                         float in_scale, float* x_out, void* workspace, size_t ws_bytes,
                         void* stream);
/* Loss L = mean((f(s x) - s (target - x))^2) into *loss (device double) and
 * its parameter gradient into grad (device, param_count floats; NULL keeps it
 * in the workspace).  Training workspace. */
nr_status nr_cnn_loss_grad(const nr_cnn_dims* d, const float* params, const float* x,
                           const float* target, float in_scale, float* grad, double* loss,
                           void* workspace, size_t ws_bytes, void* stream);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected; step >= 1). */
nr_status nr_cnn_adam(float* params, float* m, float* v, const float* grad, int64_t n,
                      int32_t step, float lr, void* stream);
/* nr_cnn_loss_grad then nr_cnn_adam with the workspace's gradient. */
nr_status nr_cnn_train_step(const nr_cnn_dims* d, float* params, float* adam_m, float* adam_v,
                            int32_t step, float lr, const float* x, const float* target,
                            float in_scale, double* loss, void* workspace, size_t ws_bytes,
                            void* stream);
/* Reads and clears the CNN workspace's status word (bounded tensor-core waits
 * that expired report NR_ERR_TIMEOUT).  Synchronises the stream. */
nr_status nr_cnn_check(void* workspace, int32_t* flags, void* stream);

/* Penalized-likelihood objective in FP64 (no reference counterpart; the
 * reference has no objective):
 *   out[0] = sum_i (ybar_i + r_i - y_i log(ybar_i + r_i)),  ybar = b exp(-FP_cos(x))
 *   out[1] = 1/2 sum_j sum_k w_jk psi(x_j - x_k)
 * out is a device pointer to 2 doubles; total = out[0] + beta * out[1]. */
nr_status nr_ostr_objective(const nr_geom* g, const nr_ostr_params* p,
                            const float* x, double* out, void* workspace,
                            size_t ws_bytes, void* stream);

/* Reads and clears the workspace's device status word (NaN/Inf detection)
 * after synchronising the stream.  *flags = 0 when clean. */
nr_status nr_ostr_check(void* workspace, size_t ws_bytes, int32_t* flags,
                        void* stream);

/* nr_ostr_project (the fused forward projection and gradient h of one subset)
 * that also returns, in data_out[0] (one device double), the subset's FP64
 * data term: the sum over its views' bins of ybar + r - y log(ybar + r), each
 * bin's term formed as in nr_ostr_objective's out[0] (whose views it sums
 * over), from the same projection that makes h.  For subset-level step
 * acceptance (the subset objective subset_num * data + beta * penalty).  No
 * counterpart in the reference, whose gold driver evaluates no objective
 * (Tomo_OSTR_gold.cpp:724-887).  The projection walks fp_batch steps per
 * gather round (the direct walk, whatever fp_stage says). */
nr_status nr_ostr_project_fp64(const nr_geom* g, const nr_ostr_params* p, const float* x,
                               int32_t subset, double* data_out, void* workspace,
                               size_t ws_bytes, void* stream);

/* The penalty alone, out[0] = nr_ostr_objective's out[1] (one device double),
 * over the workspace's partial sums.  No counterpart in the reference. */
nr_status nr_ostr_penalty(const nr_geom* g, const nr_ostr_params* p, const float* x,
                          double* out, void* workspace, size_t ws_bytes, void* stream);

/* The same three entry points under the names of the path's C-ABI contract
 * (fused sub-iteration, FP64 objective, workspace size): identical arguments
 * and behaviour.  nr_workspace_size takes the parameters as well as the
 * geometry: the workspace holds each subset's views (subset_num) and the
 * scatter counts only when has_scatter is set, so the size depends on both. */
nr_status nr_ostr_subset(const nr_geom* g, const nr_ostr_params* p, float* x, int32_t subset,
                         void* workspace, size_t ws_bytes, void* stream);
nr_status nr_objective_fp64(const nr_geom* g, const nr_ostr_params* p, const float* x,
                            double* out, void* workspace, size_t ws_bytes, void* stream);
nr_status nr_workspace_size(const nr_geom* g, const nr_ostr_params* p, size_t* bytes);

/* Test hook for the bounded waits.  The kernels that wait on mbarriers (the
 * TMA-fed update tile, the TMA-staged projection, the tensor-core
 * convolutions) read the second status word of their workspace (an OSTR
 * workspace, or the CNN's): with wait_index >= 0 set there, the wait number
 * wait_index of every block (the update's ring plane, the projection's slab,
 * the convolution CTA's tile) reports that it gave up once it has in fact
 * succeeded.  Nothing is in flight at that point, so the failure path runs
 * as it would after a real expiry -- the block flags NR_FLAG_TIMEOUT, stops
 * issuing copies and MMAs, drains, releases its tensor memory -- and the
 * next check returns NR_ERR_TIMEOUT.  wait_index < 0 turns the hook off;
 * nr_ostr_check also clears it on an OSTR workspace after a flagged run.
 * Enqueued on the stream.  No counterpart in the reference, which ignores
 * CUDA errors (Tomo_OSTR_gold.cpp:460-462). */
nr_status nr_test_expire_wait(void* workspace, int32_t wait_index, void* stream);

/* The penalty of nr_ostr_objective (out[1] there) computed without any
 * workspace, into out[0] (one device double), for callers that may not
 * allocate device memory: a scanner-side reconstruction service whose memory
 * is fixed at start-up, or a host framework that owns every device buffer.
 * No counterpart in the reference.  It allocates nothing: its scratch (the
 * per-block partial sums) is a file-scope device array of NR_STATIC_PARTIALS
 * = 2^18 doubles (2 MiB, held on every GPU that loads the library until the
 * process exits), which limits the volume to 2^18 blocks of 32 x 4 voxel
 * columns per plane, i.e. ceil(nx/32) * ceil(ny/4) * nz <= 262144
 * (1024x512x64 fits); larger volumes return NR_ERR_WORKSPACE.  The first call
 * on each device looks up the array's device address (cudaGetSymbolAddress)
 * with that device current; make that first call before any stream capture.
 * The address is cached with the id of the CUDA context it belongs to, and
 * looked up again when a call comes from a new context of that device (after
 * cudaDeviceReset); make the first call after a reset outside a capture too.
 * A failed lookup returns NR_ERR_CUDA and leaves CUDA's last error clear.
 * Every call shares the one array: calls that overlap on the GPU (other
 * streams, other host threads) race on it and must be serialised by the
 * caller.  Each call overwrites the partials it uses, so nothing carries over. */
nr_status nr_penalty_fp64_static(const nr_geom* g, const float* x, int32_t potential,
                                 float delta, double* out, void* stream);

/* ---------------------------------------------------------------------------
 * SART / OS-SART family on the same projectors.
 * Reference-shaped operators first (drop-in for the SART launch wrappers),
 * then the device-resident OS-SART loop (the reference's Recon_Method 3 is an
 * empty placeholder, Tomo_OSTR_gold.cpp:1523-1525).
 * ------------------------------------------------------------------------- */

/* prj_est[(a-a0)][i][j] = Siddon line integral of x (times cos(theta) when
 * use_cos) and normprj[(a-a0)][i][j] = the ray's in-volume chord, from one
 * walk, views index[a], a in [a0,a1).  Rays that miss the volume leave both
 * untouched.  Replaces fprojectCB_1R_GPU_SART (use_cos = 0,
 * Tomo_OSTR.cu:2278-2304; kernel :1177) and fprojectCB_1R_GPU_SART_cos
 * (use_cos = 1, :2306-2332; kernel :1245). */
nr_status nr_fp_sart(const nr_geom* g, const float* x, float* prj_est, float* normprj,
                     const float* angles, const int32_t* index, int32_t a0, int32_t a1,
                     int32_t use_cos, void* stream);

/* Detector layouts a projector can write. */
enum {
    NR_LAYOUT_IJ = 0,      /* [view][i][j], j fastest: the 1R projectors' layout           */
    NR_LAYOUT_JI = 1       /* [view][j][i], i fastest: the scanner files' layout            */
};

/* 2 x 2 super-sampled projection: per bin, the mean of the line integrals of
 * the four sub-rays through the sub-bin centres x_d0 + (2i+a+0.5) Bsize_x/2,
 * y_d0 + (2j+b+0.5) Bsize_y/2 (a, b in {0, 1}), sub-rays that miss the volume
 * counting 0, summed in the order (((s00 + s10) + s01) + s11) / 4, times
 * cos(theta) when use_cos.  prj gets every bin of views index[a], a in
 * [a0,a1), in `layout`; sub, if not NULL, gets the sub-ray sums
 * [view][2 BINSy][2 BINSx] (missed sub-rays untouched).  Replaces
 * fprojectCB1_4R_GPU_SART (Tomo_OSTR.cu:2398-2433; kernels :1453, :1517),
 * fixed: the reference does not compile (nBatchBINSx_4R / PRJ_*_4R are
 * undefined) and its merge never assigns the fourth sub-ray's index
 * (:1545-1547).  Its drop-in is use_cos = 0, layout = NR_LAYOUT_JI (the layout
 * its merge writes); the sub-ray buffer it needs is optional here. */
nr_status nr_fp_4r(const nr_geom* g, const float* x, float* prj, float* sub,
                   const float* angles, const int32_t* index, int32_t a0, int32_t a1,
                   int32_t use_cos, int32_t layout, void* stream);

/* diff[k] = (prj[k] - prj_est[k]) / normprj[k] where normprj[k] != 0, else 0,
 * for k < n (n = (a1-a0)*BINSx*BINSy for the reference's view range).
 * Replaces SART_prj_diff (Tomo_OSTR.cu:2537-2558; kernel :2145). */
nr_status nr_sart_prj_diff(float* diff, const float* prj, const float* prj_est,
                           const float* normprj, int64_t n, void* stream);

/* OS-SART update of x in place from the [view][i][j] difference of views
 * index[a], a in [a0,a1): per voxel, u = sum of the depth-weighted bilinear
 * back projection, s = the same of a detector of ones (the sensitivity);
 * x = max(0, x + lambda (u + beta prior) / s), both terms 0 where s = 0.
 * prior == NULL replaces bprojectCB_4B_GPU_SART (Tomo_OSTR.cu:2460-2495;
 * kernel :1737); otherwise bprojectCB_4B_GPU_SART_R (:2497-2535; kernel
 * :1938).  Note the sign: the reference ADDS beta * prior, and prior (below)
 * is the penalty gradient, so a smoothing penalty takes beta < 0. */
nr_status nr_bp_ossart(const nr_geom* g, float* x, const float* diff, const float* prior,
                       const int32_t* index, const float* angles, int32_t a0, int32_t a1,
                       float lambda, float beta, void* stream);

/* prior += sum over the 26 neighbours of (x_j - x_k) / sqrt(1 + ((x_j - x_k)/delta)^2)
 * / dist_k, dist_k the plain neighbour distance (no z ratio); out-of-volume
 * neighbours count as t = 0.  delta == 0 returns NR_ERR_BAD_ARGUMENT (the
 * reference exits).  Replaces prior_GPU_SART (Tomo_OSTR.cu:2249-2276;
 * G_Huber_prior :258-325). */
nr_status nr_prior_sart(const nr_geom* g, float* prior, const float* x, float delta,
                        void* stream);

/* SART input from a transmission scan: line[k] = log(blank[k] / (prj[k] - scat[k]))
 * where prj - scat > 0 and blank > 0, else 0; scat may be NULL.  The log
 * transform of the reference's MATLAB examples (ReconDBT/gen_dbtproj_example.m:113);
 * the CUDA code takes line integrals as given. */
nr_status nr_sart_line_integrals(float* line, const float* prj, const float* blank,
                                 const float* scat, int64_t n, void* stream);

typedef struct nr_sart_params {
    int32_t subset_num;        /* M; must divide n_angles, n_angles/M <= 32      */
    int32_t use_cos;           /* 1: the _cos projector, 0: plain line integrals */
    int32_t regularized;       /* 1: prior_GPU_SART + backprj_OSSART_R           */
    int32_t fp_batch;          /* Siddon steps per gather round: 2, 4, 8 (0 = 4) */
    int32_t upd_planes;        /* z planes per update block: 8, 16, 32 (0 = 16) */
    float lambda;              /* relaxation                                     */
    float beta;                /* prior weight (regularized only; see the sign note above) */
    float delta;               /* hyperbola scale, != 0 (regularized only)      */
    int32_t supersample;       /* 1: the 2 x 2 sub-ray projector of nr_fp_4r (and its
                                  mean chord as normprj); 0: one ray per bin      */
} nr_sart_params;

/* Bytes of workspace the OS-SART loop needs. */
nr_status nr_sart_workspace_size(const nr_geom* g, const nr_sart_params* p, size_t* bytes);

/* Load the line integrals ([view][i][j], ORIGINAL view order) into the
 * workspace in subset order and trace every ray's chord (normprj) once. */
nr_status nr_sart_setup(const nr_geom* g, const nr_sart_params* p, const float* angles,
                        const float* line, void* workspace, size_t ws_bytes, void* stream);

/* n_iters iterations (M sub-iterations each, subset-major view order as the
 * OSTR driver, Tomo_OSTR_gold.cpp:628-642) on x in place.  Per sub-iteration:
 * diff = (p - FP_SART(x)) / normprj (0 where normprj = 0) over the subset, then
 * the OS-SART update above with the prior of the current x.  The status word
 * (NaN/Inf) is read with nr_ostr_check on this workspace. */
nr_status nr_sart_iterate(const nr_geom* g, const nr_sart_params* p, float* x,
                          int32_t n_iters, void* workspace, size_t ws_bytes, void* stream);

/* The two halves of sub-iteration `subset`: the fused projection and
 * difference into the workspace, then x_out = the OS-SART update of x
 * (x_out != x).  nr_sart_subiter = project + update + copy back. */
nr_status nr_sart_project(const nr_geom* g, const nr_sart_params* p, const float* x,
                          int32_t subset, void* workspace, size_t ws_bytes, void* stream);
nr_status nr_sart_update(const nr_geom* g, const nr_sart_params* p, const float* x,
                         float* x_out, int32_t subset, void* workspace, size_t ws_bytes,
                         void* stream);

/* One sub-iteration for subset a (0 <= a < M), x in place. */
nr_status nr_sart_subiter(const nr_geom* g, const nr_sart_params* p, float* x,
                          int32_t subset, void* workspace, size_t ws_bytes, void* stream);

/* nr_sart_iterate captured once into a CUDA graph on `stream` (x and the
 * workspace are bound into it); launch and destroy it with
 * nr_ostr_graph_launch / nr_ostr_graph_destroy. */
nr_status nr_sart_graph_create(const nr_geom* g, const nr_sart_params* p, float* x,
                               int32_t n_iters, void* workspace, size_t ws_bytes,
                               void* stream, void** graph);

/* Workspace sections a caller may read (device pointer + byte size). */
enum {
    NR_SART_WS_LINE = 0,   /* float[A][BINSy][BINSx]: line integrals, subset order   */
    NR_SART_WS_NORM = 1,   /* float[A][BINSy][BINSx]: chord per ray, subset order    */
    NR_SART_WS_DIFF = 2,   /* float[Vs][BINSy][BINSx]: last subset's difference      */
    NR_SART_WS_INDEX = 3   /* int32[A]: subset-major view order                      */
};
nr_status nr_sart_workspace_section(const nr_geom* g, const nr_sart_params* p,
                                    int32_t section, void* workspace, size_t ws_bytes,
                                    void** ptr, size_t* bytes);

/* ---------------------------------------------------------------------------
 * Dual-energy weighted subtraction (syncrecon.m:1-41): post-processing of a
 * high-energy (he) and a low-energy (le) reconstruction on the device.
 * ------------------------------------------------------------------------- */

/* For each of n_weights (1..16) weights w_k (host array of doubles):
 * d[k][i] = float(double(he[i]) - double(le[i]) * w_k), i < n, rounded in
 * double exactly as MATLAB's `d = he - le*weight` on the float32 volumes it
 * reads (syncrecon.m:28).  mask_level >= 0 first zeroes he and le where
 * he <= mask_level (the imbinarize(he, graythresh(he)) mask of :7-8, applied
 * in its commented-out :21-22); mask_level < 0 uses no mask.  If hist is not
 * NULL it gets hist[k][b] = the number of i in [hist_begin, hist_begin +
 * hist_len) whose double d_k falls in 8-bit bin b = round(255 d) saturated to
 * [0, 255] (the histogram MATLAB's entropy(d(:,:,slice)) counts, :34).
 * he, le and d 16-byte aligned; d holds n_weights * n floats. */
nr_status nr_de_subtract(const float* he, const float* le, const double* weights,
                         int32_t n_weights, int64_t n, double mask_level, float* d,
                         int64_t hist_begin, int64_t hist_len, int32_t* hist, void* stream);

/* hist[b] = the number of x[i] (i < n) in 8-bit bin b, as above (the
 * histogram of graythresh, syncrecon.m:7).  hist: 256 int32 on the device. */
nr_status nr_hist8(const float* x, int64_t n, int32_t* hist, void* stream);

/* Host functions on a 256-bin histogram in HOST memory (no GPU work):
 * Shannon entropy in bits of `count` values (MATLAB's entropy), and Otsu's
 * threshold as a level in [0, 1] (graythresh: bin of maximal between-class
 * variance, the mean index of ties, / 255; 0 when the maximum is not finite). */
nr_status nr_hist_entropy(const int32_t* hist, int64_t count, double* entropy);
nr_status nr_otsu_level(const int32_t* hist, double* level);

/* Library version string. */
const char* nr_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NRGB300_H */
