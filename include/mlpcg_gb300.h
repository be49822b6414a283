/*
 * mlpcg_gb300.h -- C ABI of the GB300 (sm_103a) neural-preconditioned CG library.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*, i.e. a cudaStream_t; NULL = legacy default stream), launches
 * asynchronously on that stream and returns an int status (0 = ok, negative =
 * argument error, see MLPCG_ERR_*).  A failing call leaves a message readable
 * through mlpcg_last_error() (thread-local).  No entry point allocates device
 * memory: where scratch space is needed the caller passes a workspace whose
 * size is given by the matching *_workspace() query.  Nothing is retained
 * between calls except the opaque solver objects created by
 * mlpcg_solver_create(), which hold host-side state only.
 *
 * Grid layout: a field on an N1 x N2 x N3 grid is stored contiguously with
 * N3 fastest (index (i*N2 + j)*N3 + k), batches of B fields back to back.
 * That is the layout of the reference's (B, 1, N1, N2, N3) tensors.
 * "padded" inputs are (N1+2) x (N2+2) x (N3+2) arrays whose outer layer is
 * read as the halo, exactly like the F.pad'ed tensors the reference's
 * extension modules receive (sm_model_3d.py:24-26).
 *
 * Reference file citations are paths inside kai-lan/MLPCG.
 */
#ifndef MLPCG_GB300_H
#define MLPCG_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
#define MLPCG_OK               0
#define MLPCG_ERR_ARG         -1  /* null pointer, bad enum, negative size   */
#define MLPCG_ERR_SHAPE       -2  /* sizes the operation does not support    */
#define MLPCG_ERR_ALIGN       -3  /* pointer / stride alignment violated     */
#define MLPCG_ERR_WORKSPACE   -4  /* workspace too small                     */
#define MLPCG_ERR_CUDA        -5  /* a CUDA runtime call failed              */
#define MLPCG_ERR_UNSUPPORTED -6  /* dtype / mode combination not provided   */

/* ---- element types -------------------------------------------------------- */
#define MLPCG_F32  0
#define MLPCG_BF16 1
#define MLPCG_F64  2

/* ---- cell flags (lib/read_data.py:13-16) ---------------------------------- */
#define MLPCG_BOUNDARY 0
#define MLPCG_SOLID    1
#define MLPCG_FLUID    2
#define MLPCG_AIR      3

/* Message of the last failing call on this host thread ("" if none). */
const char *mlpcg_last_error(void);
/* ABI version of the loaded library. */
int mlpcg_abi_version(void);

/* =========================================================================
 * Stencil-coefficient generation and application (the two halves of the
 * reference's sm_block_3d / sm_block_trans_3d kernels).
 * ========================================================================= */

/*
 * K_p(q) = bias[p] + sum_{s<3, m,n,o<3} weight[p][s][m][n][o] * img(s, q+(m-1,n-1,o-1))
 * for the 27 taps p of every cell q (img zero outside the grid, or read from
 * the halo when image_padded).  Writes 27 planes K[p*plane_stride + cell].
 * Replaces the per-thread coefficient loop of sm_block_3d_cuda_inference_kernel
 * (torch_extension/sm_block_3d_kernel.cu:45-65), which the reference re-runs
 * on every call; here it runs once per (image, weights).
 * k_dtype: MLPCG_F32 or MLPCG_BF16.  plane_stride >= N1*N2*N3, multiple of 8.
 */
int mlpcg_stencil_gen(const float *image, int image_padded, int N1, int N2, int N3,
                      const float *weight, const float *bias,
                      void *K, int k_dtype, int64_t plane_stride, void *stream);

/*
 * transpose = 0:  y(q) = sum_p K_p(q) * x(q + off_p)           (sm_block_3d_kernel.cu:66-70)
 * transpose = 1:  y(q) = sum_p K_p(q - off_p) * x(q - off_p)   (sm_block_trans_3d_kernel.cu:45-73)
 * with off_p = (p/9-1, (p/3)%3-1, p%3-1) and x zero outside the grid (or read
 * from the halo when x_padded).  x, y hold B fields.
 * K: F32|BF16; x: F32|BF16; y: F32|BF16.
 */
int mlpcg_stencil_apply(const void *K, int k_dtype, int64_t plane_stride,
                        const void *x, int x_dtype, int x_padded,
                        void *y, int y_dtype,
                        int B, int N1, int N2, int N3, int transpose, void *stream);

/*
 * Gradient of a stencil application with respect to its coefficients, summed
 * over the batch:
 *   transpose = 0:  dK_p(q)  = sum_b g_b(q) * x_b(q + off_p)
 *   transpose = 1:  dK_p(q)  = sum_b g_b(q + off_p) * x_b(q)
 * (the cell-level factors of sm_block_3d_cuda_dwdb_fast_kernel,
 *  sm_block_3d_kernel.cu:122-229, and its transpose, sm_block_trans_3d_kernel.cu:173-289).
 * dK is F32 with 27 planes of plane_stride.
 */
int mlpcg_stencil_coeff_grad(const float *g, const float *x, int x_padded, float *dK,
                             int64_t plane_stride, int B, int N1, int N2, int N3,
                             int transpose, void *stream);

/*
 * grad_weight[p][s][m][n][o] = sum_q dK_p(q) * img(s, q+(m-1,n-1,o-1)),
 * grad_bias[p] = sum_q dK_p(q).  Deterministic two-pass reduction (no atomics).
 * Overwrites grad_weight (27*81 floats) and grad_bias (27 floats).
 * Workspace: mlpcg_stencil_wgrad_workspace(N1,N2,N3) bytes.
 */
size_t mlpcg_stencil_wgrad_workspace(int N1, int N2, int N3);
int mlpcg_stencil_wgrad(const float *dK, int64_t plane_stride,
                        const float *image, int image_padded, int N1, int N2, int N3,
                        float *grad_weight, float *grad_bias,
                        void *workspace, size_t workspace_bytes, void *stream);

/*
 * Gradient with respect to the image channels:
 *   grad_image(s, c) = sum_{p, m,n,o} weight[p][s][m][n][o] * dK_p(c - (m-1,n-1,o-1)).
 * (The reference returns no image gradient; this is the adjoint of
 * mlpcg_stencil_gen restricted to its image argument.)  Overwrites grad_image
 * (3 x N1 x N2 x N3, F32, unpadded).
 */
int mlpcg_stencil_image_grad(const float *dK, int64_t plane_stride,
                             const float *weight, float *grad_image,
                             int N1, int N2, int N3, void *stream);

/* =========================================================================
 * Reference extension ops (smblock3d / smblocktrans3d / smlinear3d)
 * ========================================================================= */

/* Workspace of mlpcg_sm_block_3d_forward/backward: one K buffer (+ reduction space). */
size_t mlpcg_sm_block_3d_workspace(int N1, int N2, int N3);

/*
 * smblock3d.inference/forward (transpose = 0) and smblocktrans3d.inference/forward
 * (transpose = 1): torch_extension/sm_block_3d.cpp:31-55,
 * sm_block_3d_kernel.cu:329-418, sm_block_trans_3d_kernel.cu:381-470.
 * image: 3 x N1 x N2 x N3 (or padded), x: B x N1 x N2 x N3 (or padded),
 * weight: 27 x 3 x 3 x 3 x 3, bias: 27, y: B x N1 x N2 x N3.  All F32.
 * Unlike the reference, any B and any N >= 1 are accepted (the reference's
 * forward asserts N3 % 2 == 0, sm_block_3d_kernel.cu:399).
 */
int mlpcg_sm_block_3d_forward(const float *image, int image_padded,
                              const float *x, int x_padded,
                              const float *weight, const float *bias, float *y,
                              int B, int N1, int N2, int N3, int transpose,
                              void *workspace, size_t workspace_bytes, void *stream);

/*
 * smblock3d.backward / smblocktrans3d.backward: sm_block_3d.cpp:57-69,
 * sm_block_3d_kernel.cu:420-484, sm_block_trans_3d_kernel.cu:472-535.
 * Returns grad_x (B x N), grad_weight (27 x 81), grad_bias (27), F32, for any B
 * (the reference's dx kernels are only correct for B = 128,
 * sm_block_3d_kernel.cu:18-20).  grad_image may be NULL; when given it
 * receives d/d image (3 x N, unpadded), which the reference does not provide.
 */
int mlpcg_sm_block_3d_backward(const float *grad_out,
                               const float *image, int image_padded,
                               const float *x, int x_padded,
                               const float *weight, const float *bias,
                               float *grad_x, float *grad_weight, float *grad_bias,
                               float *grad_image,
                               int B, int N1, int N2, int N3, int transpose,
                               void *workspace, size_t workspace_bytes, void *stream);

/*
 * smlinear3d.inference/forward: sm_linear_3d.cpp:25-47, sm_linear_3d_kernel.cu:152-227.
 *   y[s][k][l][o] = (1/(N1 N2 N3)) sum_q img(s, q + (k-1,l-1,o-1))   (81 values, img zero outside)
 *   z[j]          = sum_i weight[j][i] * y[i] + bias[j]             for j < nlin
 * image: 3 x N1 x N2 x N3 unpadded, weight: nlin x 81, bias: nlin, z: nlin, y: 81, F32.
 * nlin > 1 evaluates several linear blocks on one image in one pass (the
 * reference's c0/c1 blocks of one level share the image).
 * Workspace: mlpcg_sm_linear_3d_workspace(N1,N2,N3) bytes.
 */
size_t mlpcg_sm_linear_3d_workspace(int N1, int N2, int N3);
int mlpcg_sm_linear_3d_forward(const float *image, int N1, int N2, int N3,
                               const float *weight, const float *bias, int nlin,
                               float *z, float *y,
                               void *workspace, size_t workspace_bytes, void *stream);

/*
 * smlinear3d.backward: sm_linear_3d_kernel.cu:229-238.
 *   grad_weight[i] = y[i] * grad_out[0]   (81 values), grad_bias[0] = grad_out[0].
 */
int mlpcg_sm_linear_3d_backward(const float *grad_out, const float *y,
                                float *grad_weight, float *grad_bias, void *stream);

/*
 * Gradient of z = w.y(img) + b with respect to the image:
 *   grad_image(s, c) = grad_out * (1/N) * sum_{k,l,o : c-(k-1,l-1,o-1) in grid} w[s][k][l][o].
 * (Not provided by the reference.)  Overwrites grad_image (3 x N, F32).
 */
int mlpcg_sm_linear_3d_image_grad(const float *grad_out, const float *weight,
                                  float *grad_image, int N1, int N2, int N3, void *stream);

/* =========================================================================
 * Grid transfer between levels (ATen ops the reference calls,
 * sm_model_3d.py:206-230, 269-278)
 * ========================================================================= */

/* F.avg_pool3d(x, 2): N1,N2,N3 are the fine sizes (even); y is B x N/2. */
int mlpcg_avg_pool2(const void *x, void *y, int dtype, int B, int N1, int N2, int N3,
                    void *stream);
/* Adjoint of avg_pool2: x(fine) = y(coarse cell containing it) / 8. */
int mlpcg_avg_pool2_adjoint(const void *y, void *x, int dtype, int B, int N1, int N2, int N3,
                            void *stream);
/* F.interpolate(x, scale_factor=2, mode='trilinear', align_corners=False):
 * n1,n2,n3 are the coarse sizes; y is B x 2n. */
int mlpcg_upsample2(const void *x, void *y, int dtype, int B, int n1, int n2, int n3,
                    void *stream);
/* Adjoint of mlpcg_upsample2 (gradient of the interpolation w.r.t. its input). */
int mlpcg_upsample2_adjoint(const void *y, void *x, int dtype, int B, int n1, int n2, int n3,
                            void *stream);
/* out = c0[0]*x + c1[0]*y with c0, c1 device scalars (sm_model_3d.py:258,286). */
int mlpcg_axpby(const float *c0, const void *x, const float *c1, const void *y, void *out,
                int dtype, int64_t n, void *stream);

/* =========================================================================
 * Matrix-free 7-point Poisson operator with mixed boundaries.
 * The reference assembles it as an FP64 CSR (lib/discrete_laplacian.py:122-160,
 * lib/read_data.py:110-165) and multiplies with torch.sparse (cg_tests.py:53,80,83).
 *   (A x)(c) = d(c) x(c) - sum_{fluid face neighbours n} x(n)  for FLUID c, else 0,
 *   d(c)     = number of non-solid (FLUID or AIR) face neighbours.
 * Cells outside the grid count as solid.
 * ========================================================================= */
int mlpcg_laplacian_apply(const uint8_t *flags, const void *x, void *y, int dtype,
                          int N1, int N2, int N3, void *stream);

/* =========================================================================
 * Preconditioner plan: SmallSMModelDn3D.eval_forward (sm_model_3d.py:180-262)
 * with every block's coefficients precomputed once per (image, weights).
 * The reference re-evaluates them inside every sm_block_3d call
 * (sm_block_3d_kernel.cu:45-65) and only caches the image pyramid and c0/c1
 * (sm_model_3d.py:180-239).  Application = 2*levels+1 fused kernels:
 * restriction fused into the pre-blocks, trilinear prolongation and the
 * c0/c1 combine fused into the post-blocks.
 * ========================================================================= */
typedef struct mlpcg_precond mlpcg_precond;

/* Coefficient layouts of a plan.
 * DENSE:   27 planes per block (27 values per cell).
 * CLASSED: one word per 8-cell z-run.  A cell whose 3x3x3 image neighbourhood
 *          is a single one-hot material (solid or outside, air, fluid) has
 *          that material's constant coefficient vector; a run of 8 such cells
 *          of one material is described by the material alone, any other
 *          ("mixed") run by a record of its 27 x 8 coefficients.
 *          Bit-identical results, far less coefficient traffic on scenes
 *          made of large regions. */
#define MLPCG_COEFF_DENSE   0
#define MLPCG_COEFF_CLASSED 1

/* Host-side plan for an N1 x N2 x N3 grid (each divisible by 2^levels).
 * k_dtype / act_dtype: storage of coefficients / level activations, F32 or
 * BF16 (arithmetic is FP32).  swap_sm_order and mask have the meaning of the
 * SmallSMModelDn3D constructor arguments.  coeff_layout: MLPCG_COEFF_*
 * (levels whose z size is not a multiple of 8 always use dense planes). */
int mlpcg_precond_create(int N1, int N2, int N3, int levels, int k_dtype, int act_dtype,
                         int swap_sm_order, int mask, int coeff_layout, mlpcg_precond **out);

/* Network kinds of a plan. */
#define MLPCG_PRECOND_SM        0  /* SmallSMModelDn3D (sm_model_3d.py:164-287) */
#define MLPCG_PRECOND_SMALL_SPD 1  /* SmallSPDSMModelDn3D (sm_model_3d.py:388-444) */
#define MLPCG_PRECOND_SPD       2  /* SPDSMModelDn3D (sm_model_3d.py:290-385) */

/* Plan for the reduced symmetric network SmallSPDSMModelDn3D(levels)
 * (sm_model_3d.py:388-444; replaces its eval_forward inside the solver
 * loop): M = S^T S, S the down sweep of blocks l0[0..n-1] with average
 * pooling and the coarsest block l.  Application: the down sweep, l then
 * l_t on the coarsest level, and per level the nearest x2 / 8 prolongation,
 * c0^2 y + c1^2 u and the transposed block l0_t.  The transposed blocks'
 * coefficients are gathered from the forward blocks' (B^T has at cell q
 * the coefficient 26 - p of cell q + offset p), so no image is re-read.
 * setup's params: l0[0..n-1], l as (weight 2187, bias 27), then c0[0..n-1],
 * c1[0..n-1] as (weight 81, bias 1); mlpcg_precond_coefficients returns the
 * squares c0^2, c1^2 for this kind.  Other arguments as mlpcg_precond_create
 * (no swap / mask options: the network has none). */
int mlpcg_precond_create_spd(int N1, int N2, int N3, int levels, int k_dtype, int act_dtype, int coeff_layout,
                             mlpcg_precond **out);
/* Plan for network kind MLPCG_PRECOND_SMALL_SPD (as mlpcg_precond_create_spd)
 * or MLPCG_PRECOND_SPD: SPDSMModelDn3D(levels) (sm_model_3d.py:290-385;
 * replaces its eval_forward inside the solver loop), M = V^T V with V the
 * V-cycle of blocks l0 (down, average pooling), l (coarsest), nearest x2 / 8
 * prolongation, l1 and c0 y + c1 u (up); the application runs V, then V^T:
 * l1_t and pooling down from V's output, l_t, then per level the
 * prolongation, c0 x_l + c1 u with x_l the level's input of that down
 * sweep, and l0_t.  The transposed blocks' coefficients are gathered from
 * the forward blocks' as for the reduced network.  setup's params for
 * MLPCG_PRECOND_SPD: l0[0..n-1], l1[0..n-1], l (weight 2187, bias 27 each),
 * then c0[0..n-1], c1[0..n-1] (weight 81, bias 1) -- the layout of
 * mlpcg_precond_create's pre / post / l.  Application stages
 * (mlpcg_precond_apply_stages): 0 .. 2n as for the other networks for V,
 * 2n + 1 .. 4n + 1 the same sequence for V^T. */
int mlpcg_precond_create_kind(int N1, int N2, int N3, int levels, int kind, int k_dtype, int act_dtype,
                              int coeff_layout, mlpcg_precond **out);
/* After setup of an SPD plan (either kind): mlpcg_precond_class_counts of the
 * level's transposed blocks (l0_t / l1_t, or l_t on the coarsest level; they
 * share one class map), whose cells are uniform when their 27 neighbours
 * are; MLPCG_ERR_ARG for other plans. */
int mlpcg_precond_class_counts_transposed(const mlpcg_precond *plan, int level, int64_t *general_cells,
                                          int64_t *mixed_runs, void *stream);
/* After setup (synchronises `stream`): the number of general cells and of
 * mixed runs (records) of a classed level; -1 for both on a dense level. */
int mlpcg_precond_class_counts(const mlpcg_precond *plan, int level, int64_t *general_cells, int64_t *mixed_runs,
                               void *stream);
/* Device bytes the plan needs (caller allocates, 256-byte aligned). */
size_t mlpcg_precond_workspace(const mlpcg_precond *plan);
void mlpcg_precond_destroy(mlpcg_precond *plan);
/*
 * Builds the image pyramid, the coefficient planes of all 2*levels+1 blocks
 * and the per-level c0/c1 scalars.  image: 3 x N (F32, the [air, fluid,
 * non-solid] channels, lib/read_data.py:28-39).  params: device F32 array
 * packing, in order, pre[0..n-1], post[0..n-1], l as (weight 2187, bias 27)
 * and then c0[0..n-1], c1[0..n-1] as (weight 81, bias 1).
 */
int mlpcg_precond_setup(mlpcg_precond *plan, void *workspace, size_t workspace_bytes,
                        const float *image, const float *params, void *stream);
/*
 * z = M(r * r_scale[0]) on the fine grid (r_scale may be NULL = 1; the
 * reference feeds the network r/||r||, test.py:46).  z is F32 and zero on
 * non-fluid cells (image channel 1 == 0), which is what the reference's
 * gather of fluid cells keeps (test.py:49-50).  r 16-byte, z 32-byte aligned.
 */
int mlpcg_precond_apply(const mlpcg_precond *plan, const float *r, const float *r_scale, float *z,
                        void *stream);
/* Runs stages [first, last] of one application (stage s < n: pre-block of
 * level s; s = n: coarsest block; s > n: post-block of level 2n - s; the
 * MLPCG_PRECOND_SPD kind repeats this for V^T as stages 2n + 1 .. 4n + 1),
 * using the plan's own level buffers.  Stage 0 reads r, the last stage
 * writes z.  Used to time the kernels of an application one by one. */
int mlpcg_precond_apply_stages(const mlpcg_precond *plan, int first, int last, const float *r,
                               const float *r_scale, float *z, void *stream);
/* After applications (synchronises `stream`): *copy_failed = 1 if a tile
 * copy of the level-0 pre-block (loaded by the tensor-memory accelerator)
 * did not complete within the kernel's bounded wait -- the outputs of such
 * an application are not valid -- else 0. */
int mlpcg_precond_check(const mlpcg_precond *plan, int *copy_failed, void *stream);
/* The coarse levels of a SmallSMModelDn3D plan (no counterpart in the
 * reference, which launches every block and transfer separately): from
 * *first_level on, an application runs the pre-blocks, the coarsest block
 * and the post-blocks in one launch of one thread-block cluster of *ctas
 * CTAs, stage after stage.  *first_level = -1 (and *ctas = 0) when no two
 * coarsest levels qualify (they must all run the tiled kernels), for the
 * symmetric kinds, when the device runs no cluster of 8 or 16 CTAs, or when
 * the plan has it switched off (mlpcg_precond_set_coarse_cluster).
 * mlpcg_precond_apply_stages uses it only when [first, last] covers all of
 * its stages (first_level .. 2n - first_level). */
int mlpcg_precond_coarse_cluster(const mlpcg_precond *plan, int *first_level, int *ctas);
/* on = 1: the plan's applications run the coarse levels as one cluster
 * launch where the device and the plan allow it; on = 0 (the default): one
 * kernel per stage.  Same arithmetic, same outputs.  Off by default: on a
 * GB300 the 256^3 npsd solve takes 8.64 ms with it and 8.46 ms without (a
 * stage's tiles share 16 SMs instead of spreading over the GPU, and each
 * stage still waits on its tiles' load -> compute chain). */
int mlpcg_precond_set_coarse_cluster(mlpcg_precond *plan, int on);
/* Block schedule of the plan's applications (no counterpart in the
 * reference): a level whose tiles number at most tiles_per_sm per SM runs the
 * block kernels that load each run's coefficients up front (BF16
 * coefficients only; 0 = never; default 2).  Same outputs either way; picked
 * per device and grid by mlpcg_gb300.autotune.  A solver bound to the plan
 * picks the change up once its graph is recaptured (mlpcg_solver_set_schedule
 * recaptures it). */
int mlpcg_precond_set_small_levels(mlpcg_precond *plan, int tiles_per_sm);
/* Test knob of the bounded TMA waits (no counterpart in the reference):
 * with on != 0 the level-0 tile kernels first wait on a barrier that nothing
 * arrives on (256 polls), so the wait runs out on an ordinary copy, whose
 * completion they then wait for before leaving; the plan's applications
 * then report copy_failed.  Every call also clears the copy-failed word;
 * on = 0 restores normal waits.  Off after every mlpcg_precond_setup. */
int mlpcg_precond_set_copy_stall(mlpcg_precond *plan, int on, void *stream);
/* Sizes of level `level` (0 = finest) and whether it runs the tiled kernels
 * (z size a multiple of 8) or the general ones. */
int mlpcg_precond_level_info(const mlpcg_precond *plan, int level, int *n1, int *n2, int *n3,
                             int *fast);
/* Copies the 2*levels per-level scalars (c0[0..n-1], c1[0..n-1]) to c_out (device). */
int mlpcg_precond_coefficients(const mlpcg_precond *plan, float *c_out, void *stream);

/* =========================================================================
 * Fused solver: the iteration of npsd (cg_tests.py:189-284, the solver of
 * test.py:327-328) or npcg (cg_tests.py:26-101) run entirely on the GPU,
 * captured once as a CUDA graph whose conditional WHILE node loops until
 * convergence.  Vectors on the full grid (zero off-fluid): r, z, p, Ap FP32;
 * x and b FP64; dot products reduced in FP64; the residual recomputed as
 * r = b - A x in FP64 every true_every iterations and before convergence is
 * declared, so the reported relative residual is the FP64 true residual.
 * ========================================================================= */
typedef struct mlpcg_solver mlpcg_solver;

#define MLPCG_METHOD_NPSD 0
#define MLPCG_METHOD_NPCG 1

#define MLPCG_STATUS_RUNNING    0
#define MLPCG_STATUS_CONVERGED  1
#define MLPCG_STATUS_MAXIT      2
#define MLPCG_STATUS_BREAKDOWN  3  /* p.Ap <= 0 */
#define MLPCG_STATUS_NONFINITE  4  /* NaN / Inf met */
#define MLPCG_STATUS_COPY_FAILED 5 /* a TMA tile copy did not complete within its bounded wait */

/* The solver keeps `plan` (not owned) as its preconditioner. */
int mlpcg_solver_create(int N1, int N2, int N3, const mlpcg_precond *plan, int method,
                        int max_it, double tol, int true_every, mlpcg_solver **out);
size_t mlpcg_solver_workspace(const mlpcg_solver *solver);
void mlpcg_solver_destroy(mlpcg_solver *solver);
/* flags: N uint8 cell codes; b: N FP64 rhs (read on FLUID cells only);
 * x: N FP64, the initial guess on entry to solve and the solution after.
 * flags 4-byte, b and x 16-byte aligned (MLPCG_ERR_ALIGN otherwise). */
int mlpcg_solver_bind(mlpcg_solver *solver, void *workspace, size_t workspace_bytes,
                      const uint8_t *flags, const double *b, double *x);
/* Enqueues the solve on `stream`.  use_graph = 1: one graph launch (the graph
 * is captured on the first call and reused until the next bind); 0: plain
 * launches with a host status check per iteration. */
int mlpcg_solver_solve(mlpcg_solver *solver, int use_graph, void *stream);
/* mlpcg_solver_solve with the initial guess x0 = 0, the reference's call
 * (test.py:328 passes torch.zeros_like(rhs) to npsd): x is not read, and
 * every cell of x is written by the solve (0 off the fluid cells). */
int mlpcg_solver_solve_zero_guess(mlpcg_solver *solver, int use_graph, void *stream);
/* Synchronises `stream`, then returns iterations, status, the final relative
 * residual and (if history != NULL) max_it+1 relative residuals (host). */
int mlpcg_solver_result(const mlpcg_solver *solver, int *iterations, int *status, double *rel_res,
                        double *history, void *stream);

/* Schedule of the solver's grid-stride kernels (no counterpart in the
 * reference): `blocks` CTAs of 256 threads (0 = automatic, at most 1216),
 * picked per grid size by mlpcg_gb300.autotune.  Takes effect on the next
 * solve (the captured graph is rebuilt); batches already built keep theirs. */
int mlpcg_solver_set_schedule(mlpcg_solver *solver, int blocks);
int mlpcg_solver_get_schedule(const mlpcg_solver *solver, int *blocks_in_use);

/* Programmatic dependent launch in the captured iteration (no counterpart in
 * the reference; on by default): consecutive kernels of the loop body are
 * joined by programmatic edges, so a kernel's blocks are scheduled while its
 * predecessor's last blocks run and wait on the device for its completion
 * (measured 0.5 % faster at 256^3, 1 % at 128^3).  Results
 * are identical either way.  Takes effect on the next solve (the graph is
 * rebuilt).  Batches capture ordinary edges (measured faster with the systems'
 * chains running side by side).  If the runtime refuses such a graph, the
 * solve captures ordinary edges.
 * mlpcg_solver_dependent_edges reports the edges converted in the current
 * graph (0 before the first graph solve or with the feature off). */
int mlpcg_solver_set_dependent_launch(mlpcg_solver *solver, int on);
int mlpcg_solver_dependent_edges(const mlpcg_solver *solver, int *edges);

/* Solver products in the preconditioner (no counterpart in the reference; on
 * by default): npsd's z.Ap_recent and z.Ap_previous (cg_tests.py:226-233) or
 * npcg's r.z (cg_tests.py:54,77) are summed by the plan's level-0 post-block
 * while z is in registers, one FP64 partial per tile, and reduced in a fixed
 * order -- z is not read again.  Applies to plans of the SmallSMModelDn3D and
 * SmallSPDSMModelDn3D kinds with a TMA-staged finest level; the others sum
 * them in a separate pass.  The two
 * forms add the same products in different orders (FP64 partials either
 * way).  Takes effect on the next solve; mlpcg_solver_fused_dots reports
 * whether a bound solver uses the epilogue. */
int mlpcg_solver_set_fused_dots(mlpcg_solver *solver, int on);
int mlpcg_solver_fused_dots(const mlpcg_solver *solver, int *active);

/* Test knob of the SpMV's bounded TMA waits (no counterpart in the
 * reference), taking effect from the next solve: with on != 0 the npsd
 * SpMV's first tile wait polls a barrier that nothing arrives on (256 polls)
 * and runs out while the real copy completes, so the solve ends with
 * MLPCG_STATUS_COPY_FAILED.  A solve also ends so when the plan's tile copies
 * failed (mlpcg_precond_set_copy_stall).  on = 0 restores normal waits. */
int mlpcg_solver_set_copy_stall(mlpcg_solver *solver, int on);

/* Many systems in one launch (no counterpart in the reference, whose solver
 * takes one system at a time): `count` (<= 64) bound solvers, each with its
 * own grid size, plan, method, tolerance and max_it, solved together by one
 * graph launch whose conditional WHILE node runs while any system is running;
 * inside an iteration every system's kernels form a parallel branch and
 * return at once for a system that has stopped (per-system convergence
 * masks).  Each system's result is read with mlpcg_solver_result.  The graph
 * is built on the first mlpcg_batch_solve; a solver must not be rebound while
 * it belongs to a batch. */
typedef struct mlpcg_batch mlpcg_batch;
int mlpcg_batch_create(mlpcg_solver *const *solvers, int count, mlpcg_batch **out);
int mlpcg_batch_solve(mlpcg_batch *batch, void *stream);
void mlpcg_batch_destroy(mlpcg_batch *batch);

/* Image channels [air, fluid, non-solid] (F32, 3 x N) from cell flags
 * (convert_to_binary_images, lib/read_data.py:28-39). */
int mlpcg_flags_to_image(const uint8_t *flags, float *image, int64_t n, void *stream);

/* Fluid-DOF vectors: the values of the fluid cells in flat cell order, the
 * compressed vectors the reference's solvers take and return (test.py:38-50,
 * lib/read_data.py:110-165).  mlpcg_fluid_order fills `order` (device, uint32,
 * mlpcg_fluid_order_entries(n) entries) from the flags; scatter writes a
 * fluid-DOF vector of m values onto the grid (0 off the fluid cells), gather
 * reads the grid's fluid cells into one; m is the vector's capacity (fluid
 * cells beyond it are read as 0 / not written).  Recompute the order when the
 * flags change. */
size_t mlpcg_fluid_order_entries(int64_t n);
int mlpcg_fluid_order(const uint8_t *flags, int64_t n, uint32_t *order, void *stream);
int mlpcg_scatter_fluid(const double *fluid_values, int64_t m, const uint8_t *flags, const uint32_t *order,
                        int64_t n, double *grid, void *stream);
int mlpcg_gather_fluid(const double *grid, const uint8_t *flags, const uint32_t *order, int64_t n,
                       double *fluid_values, int64_t m, void *stream);
/* *mapped = 1 when ptr lies in page-locked host memory allocated or registered
 * through CUDA (cudaHostAlloc / cudaMallocHost / cudaHostRegister) that kernels
 * reach at the same address, else 0.  Such a buffer may be passed as the
 * fluid-DOF vector of mlpcg_scatter_fluid / mlpcg_gather_fluid: the kernel then
 * reads or writes it over the host link itself, with no staging copy (the
 * caller keeps the host buffer alive and untouched until the stream reaches
 * the call).  A scatter from such memory runs on two CTAs per SM, so that it
 * leaves room for kernels of other streams while it waits on the link.  No
 * counterpart in the reference. */
int mlpcg_host_mapped(const void *ptr, int *mapped);

/* =========================================================================
 * Reductions
 * ========================================================================= */

/* out[0] (FP64, device) = sum_i x[i] * y[i], deterministic (fixed-order
 * FP64 block partials).  dtype F32|BF16|F64.  Replaces the torch dot / norm
 * calls of cg_tests.py:32,55-56,228,245.  Workspace: mlpcg_dot_workspace(n). */
size_t mlpcg_dot_workspace(int64_t n);
int mlpcg_dot(const void *x, const void *y, int dtype, int64_t n, double *out,
              void *workspace, size_t workspace_bytes, void *stream);

/*
 * mlpcg_dot without a workspace (no counterpart in the reference).  For
 * callers that cannot allocate device memory: real-time loops that must not
 * enter an allocator (its latency is unbounded), and host runtimes or
 * plug-in hosts that own all device memory through their own arena and give
 * a library only the buffers of its inputs and outputs.
 * The block partial sums live in a 64 KiB file-scope device array of this
 * library (one partial per 2048 elements), so n <= 16,777,216; larger n is
 * rejected with MLPCG_ERR_SHAPE and a message.  It calls no cudaMalloc,
 * cudaFree or allocating routine.  The first call on each device looks up
 * the array's device address (cudaGetSymbolAddress, with that device
 * current): make that first call before any stream capture.  Every call
 * shares the one array, so calls that overlap on the GPU (different streams
 * without ordering) race; nothing in it needs clearing between calls, since
 * each call writes every partial it reads.  Every GPU that loads the library
 * holds the 64 KiB until the process exits.
 */
int mlpcg_dot_noalloc(const void *x, const void *y, int dtype, int64_t n, double *out, void *stream);

#ifdef __cplusplus
}
#endif

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#endif /* MLPCG_GB300_H */
