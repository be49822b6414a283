// extern "C" entry points: argument validation, workspace carving, dispatch
// to the launchers of stencil.cu / gridops.cu.
#include <stdarg.h>
#include "common.cuh"

namespace mlpcg {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
void clear_error() { g_err[0] = 0; }

// launchers (stencil.cu)
int launch_stencil_gen(const float *, int, int, int, int, const float *, const float *, void *, int,
                       int64_t, cudaStream_t);
int launch_stencil_apply(const void *, int, int64_t, const void *, int, int, void *, int, int, int,
                         int, int, int, cudaStream_t);
int launch_coeff_grad(const float *, const float *, int, float *, int64_t, int, int, int, int, int,
                      cudaStream_t);
size_t wgrad_workspace(int, int, int);
int launch_wgrad(const float *, int64_t, const float *, int, int, int, int, float *, float *, void *,
                 size_t, cudaStream_t);
int launch_image_grad(const float *, int64_t, const float *, float *, int, int, int, cudaStream_t);
// launchers (gridops.cu)
int launch_avg_pool2(const void *, void *, int, int, int, int, int, cudaStream_t);
int launch_avg_pool2_adjoint(const void *, void *, int, int, int, int, int, cudaStream_t);
int launch_upsample2(const void *, void *, int, int, int, int, int, cudaStream_t);
int launch_upsample2_adjoint(const void *, void *, int, int, int, int, int, cudaStream_t);
int launch_axpby(const float *, const void *, const float *, const void *, void *, int, int64_t,
                 cudaStream_t);
size_t linear_workspace();
int launch_linear_forward(const float *, int, int, int, const float *, const float *, int, float *,
                          float *, void *, size_t, cudaStream_t);
int launch_linear_backward(const float *, const float *, float *, float *, cudaStream_t);
int launch_linear_image_grad(const float *, const float *, float *, int, int, int, cudaStream_t);
int launch_laplacian(const uint8_t *, const void *, void *, int, int, int, int, cudaStream_t);
int launch_flags_to_image(const uint8_t *, float *, int64_t, cudaStream_t);
int64_t fluid_blocks(int64_t n);
int launch_fluid_order(const uint8_t *, int64_t, uint32_t *, cudaStream_t);
int launch_scatter_fluid(const double *, int64_t, const uint8_t *, const uint32_t *, int64_t, double *, cudaStream_t);
int launch_gather_fluid(const double *, const uint8_t *, const uint32_t *, int64_t, double *, int64_t, cudaStream_t);
// launchers (blas.cu)
size_t dot_workspace(int64_t);
int launch_dot(const void *, const void *, int, int64_t, double *, void *, size_t, cudaStream_t);

// K planes of the op-level entry points: stride rounded up to 64 cells.
static inline int64_t plane_stride_for(int n1, int n2, int n3) {
  const int64_t n = cells(n1, n2, n3);
  return (n + 63) / 64 * 64;
}
static inline size_t align256(size_t b) { return (b + 255) / 256 * 256; }

static int check_dims(int n1, int n2, int n3) {
  MLPCG_REQUIRE(n1 >= 1 && n2 >= 1 && n3 >= 1, MLPCG_ERR_SHAPE, "grid sizes must be >= 1 (got %d %d %d)",
                n1, n2, n3);
  MLPCG_REQUIRE(cells(n1 + 2, n2 + 2, n3 + 2) < ((int64_t)1 << 40), MLPCG_ERR_SHAPE, "grid too large");
  return MLPCG_OK;
}

}  // namespace mlpcg

using namespace mlpcg;

#define CHECK_PTR(p) MLPCG_REQUIRE((p) != nullptr, MLPCG_ERR_ARG, "%s must not be NULL", #p)
#define RETURN_IF(expr) do { int _r = (expr); if (_r != MLPCG_OK) return _r; } while (0)

extern "C" {

const char *mlpcg_last_error(void) { return g_err; }
int mlpcg_abi_version(void) { return 1; }

int mlpcg_stencil_gen(const float *image, int image_padded, int N1, int N2, int N3,
                      const float *weight, const float *bias, void *K, int k_dtype,
                      int64_t plane_stride, void *stream) {
  clear_error();
  CHECK_PTR(image); CHECK_PTR(weight); CHECK_PTR(bias); CHECK_PTR(K);
  RETURN_IF(check_dims(N1, N2, N3));
  MLPCG_REQUIRE(k_dtype == MLPCG_F32 || k_dtype == MLPCG_BF16, MLPCG_ERR_UNSUPPORTED,
                "stencil_gen: K dtype must be F32 or BF16");
  MLPCG_REQUIRE(plane_stride >= cells(N1, N2, N3) && plane_stride % 8 == 0, MLPCG_ERR_ARG,
                "stencil_gen: plane_stride %lld must be >= N1*N2*N3 and a multiple of 8",
                (long long)plane_stride);
  return launch_stencil_gen(image, image_padded ? 1 : 0, N1, N2, N3, weight, bias, K, k_dtype,
                            plane_stride, as_stream(stream));
}

int mlpcg_stencil_apply(const void *K, int k_dtype, int64_t plane_stride, const void *x, int x_dtype,
                        int x_padded, void *y, int y_dtype, int B, int N1, int N2, int N3,
                        int transpose, void *stream) {
  clear_error();
  CHECK_PTR(K); CHECK_PTR(x); CHECK_PTR(y);
  RETURN_IF(check_dims(N1, N2, N3));
  MLPCG_REQUIRE(B >= 1 && B <= 65535, MLPCG_ERR_SHAPE, "stencil_apply: batch %d out of [1, 65535]", B);
  MLPCG_REQUIRE((k_dtype == MLPCG_F32 || k_dtype == MLPCG_BF16) &&
                    (x_dtype == MLPCG_F32 || x_dtype == MLPCG_BF16) &&
                    (y_dtype == MLPCG_F32 || y_dtype == MLPCG_BF16),
                MLPCG_ERR_UNSUPPORTED, "stencil_apply: dtypes must be F32 or BF16");
  MLPCG_REQUIRE(plane_stride >= cells(N1, N2, N3), MLPCG_ERR_ARG, "stencil_apply: plane_stride too small");
  return launch_stencil_apply(K, k_dtype, plane_stride, x, x_dtype, x_padded ? 1 : 0, y, y_dtype, B, N1,
                              N2, N3, transpose ? 1 : 0, as_stream(stream));
}

int mlpcg_stencil_coeff_grad(const float *g, const float *x, int x_padded, float *dK,
                             int64_t plane_stride, int B, int N1, int N2, int N3, int transpose,
                             void *stream) {
  clear_error();
  CHECK_PTR(g); CHECK_PTR(x); CHECK_PTR(dK);
  RETURN_IF(check_dims(N1, N2, N3));
  MLPCG_REQUIRE(B >= 1, MLPCG_ERR_SHAPE, "coeff_grad: batch must be >= 1");
  MLPCG_REQUIRE(plane_stride >= cells(N1, N2, N3), MLPCG_ERR_ARG, "coeff_grad: plane_stride too small");
  return launch_coeff_grad(g, x, x_padded ? 1 : 0, dK, plane_stride, B, N1, N2, N3, transpose ? 1 : 0,
                           as_stream(stream));
}

size_t mlpcg_stencil_wgrad_workspace(int N1, int N2, int N3) { return wgrad_workspace(N1, N2, N3); }

int mlpcg_stencil_wgrad(const float *dK, int64_t plane_stride, const float *image, int image_padded,
                        int N1, int N2, int N3, float *grad_weight, float *grad_bias, void *workspace,
                        size_t workspace_bytes, void *stream) {
  clear_error();
  CHECK_PTR(dK); CHECK_PTR(image); CHECK_PTR(grad_weight); CHECK_PTR(grad_bias); CHECK_PTR(workspace);
  RETURN_IF(check_dims(N1, N2, N3));
  return launch_wgrad(dK, plane_stride, image, image_padded ? 1 : 0, N1, N2, N3, grad_weight, grad_bias,
                      workspace, workspace_bytes, as_stream(stream));
}

int mlpcg_stencil_image_grad(const float *dK, int64_t plane_stride, const float *weight,
                             float *grad_image, int N1, int N2, int N3, void *stream) {
  clear_error();
  CHECK_PTR(dK); CHECK_PTR(weight); CHECK_PTR(grad_image);
  RETURN_IF(check_dims(N1, N2, N3));
  return launch_image_grad(dK, plane_stride, weight, grad_image, N1, N2, N3, as_stream(stream));
}

// ---- op-level -----------------------------------------------------------------

size_t mlpcg_sm_block_3d_workspace(int N1, int N2, int N3) {
  if (N1 < 1 || N2 < 1 || N3 < 1) return 0;
  const int64_t ps = plane_stride_for(N1, N2, N3);
  // forward: K (F32); backward: K + dK (F32) + wgrad partials
  return 2 * align256((size_t)27 * ps * sizeof(float)) + align256(wgrad_workspace(N1, N2, N3));
}

int mlpcg_sm_block_3d_forward(const float *image, int image_padded, const float *x, int x_padded,
                              const float *weight, const float *bias, float *y, int B, int N1, int N2,
                              int N3, int transpose, void *workspace, size_t workspace_bytes,
                              void *stream) {
  clear_error();
  CHECK_PTR(image); CHECK_PTR(x); CHECK_PTR(weight); CHECK_PTR(bias); CHECK_PTR(y); CHECK_PTR(workspace);
  RETURN_IF(check_dims(N1, N2, N3));
  MLPCG_REQUIRE(B >= 1 && B <= 65535, MLPCG_ERR_SHAPE, "sm_block_3d: batch %d out of [1, 65535]", B);
  const int64_t ps = plane_stride_for(N1, N2, N3);
  const size_t need = align256((size_t)27 * ps * sizeof(float));
  MLPCG_REQUIRE(workspace_bytes >= need, MLPCG_ERR_WORKSPACE,
                "sm_block_3d forward workspace too small: %zu < %zu", workspace_bytes, need);
  cudaStream_t st = as_stream(stream);
  float *K = (float *)workspace;
  RETURN_IF(launch_stencil_gen(image, image_padded ? 1 : 0, N1, N2, N3, weight, bias, K, MLPCG_F32, ps, st));
  return launch_stencil_apply(K, MLPCG_F32, ps, x, MLPCG_F32, x_padded ? 1 : 0, y, MLPCG_F32, B, N1, N2,
                              N3, transpose ? 1 : 0, st);
}

int mlpcg_sm_block_3d_backward(const float *grad_out, const float *image, int image_padded,
                               const float *x, int x_padded, const float *weight, const float *bias,
                               float *grad_x, float *grad_weight, float *grad_bias, float *grad_image,
                               int B, int N1, int N2, int N3, int transpose, void *workspace,
                               size_t workspace_bytes, void *stream) {
  clear_error();
  CHECK_PTR(grad_out); CHECK_PTR(image); CHECK_PTR(x); CHECK_PTR(weight); CHECK_PTR(bias);
  CHECK_PTR(grad_x); CHECK_PTR(grad_weight); CHECK_PTR(grad_bias); CHECK_PTR(workspace);
  RETURN_IF(check_dims(N1, N2, N3));
  MLPCG_REQUIRE(B >= 1 && B <= 65535, MLPCG_ERR_SHAPE, "sm_block_3d: batch %d out of [1, 65535]", B);
  MLPCG_REQUIRE(!(grad_image && image_padded), MLPCG_ERR_UNSUPPORTED,
                "sm_block_3d backward: grad_image needs an unpadded image");
  const size_t need = mlpcg_sm_block_3d_workspace(N1, N2, N3);
  MLPCG_REQUIRE(workspace_bytes >= need, MLPCG_ERR_WORKSPACE,
                "sm_block_3d backward workspace too small: %zu < %zu", workspace_bytes, need);
  cudaStream_t st = as_stream(stream);
  const int64_t ps = plane_stride_for(N1, N2, N3);
  const size_t kbytes = align256((size_t)27 * ps * sizeof(float));
  float *K = (float *)workspace;
  float *dK = (float *)((char *)workspace + kbytes);
  void *wg = (char *)workspace + 2 * kbytes;
  RETURN_IF(launch_stencil_gen(image, image_padded ? 1 : 0, N1, N2, N3, weight, bias, K, MLPCG_F32, ps, st));
  // dx: adjoint of the application with the same coefficients
  RETURN_IF(launch_stencil_apply(K, MLPCG_F32, ps, grad_out, MLPCG_F32, 0, grad_x, MLPCG_F32, B, N1, N2, N3,
                                 transpose ? 0 : 1, st));
  RETURN_IF(launch_coeff_grad(grad_out, x, x_padded ? 1 : 0, dK, ps, B, N1, N2, N3, transpose ? 1 : 0, st));
  RETURN_IF(launch_wgrad(dK, ps, image, image_padded ? 1 : 0, N1, N2, N3, grad_weight, grad_bias, wg,
                         workspace_bytes - 2 * kbytes, st));
  if (grad_image) RETURN_IF(launch_image_grad(dK, ps, weight, grad_image, N1, N2, N3, st));
  return MLPCG_OK;
}

size_t mlpcg_sm_linear_3d_workspace(int N1, int N2, int N3) {
  (void)N1; (void)N2; (void)N3;
  return linear_workspace();
}

int mlpcg_sm_linear_3d_forward(const float *image, int N1, int N2, int N3, const float *weight,
                               const float *bias, int nlin, float *z, float *y, void *workspace,
                               size_t workspace_bytes, void *stream) {
  clear_error();
  CHECK_PTR(image); CHECK_PTR(weight); CHECK_PTR(bias); CHECK_PTR(z); CHECK_PTR(workspace);
  RETURN_IF(check_dims(N1, N2, N3));
  MLPCG_REQUIRE(nlin >= 1 && nlin <= 128, MLPCG_ERR_ARG, "sm_linear_3d: nlin %d out of [1, 128]", nlin);
  return launch_linear_forward(image, N1, N2, N3, weight, bias, nlin, z, y, workspace, workspace_bytes,
                               as_stream(stream));
}

int mlpcg_sm_linear_3d_backward(const float *grad_out, const float *y, float *grad_weight,
                                float *grad_bias, void *stream) {
  clear_error();
  CHECK_PTR(grad_out); CHECK_PTR(y); CHECK_PTR(grad_weight); CHECK_PTR(grad_bias);
  return launch_linear_backward(grad_out, y, grad_weight, grad_bias, as_stream(stream));
}

int mlpcg_sm_linear_3d_image_grad(const float *grad_out, const float *weight, float *grad_image,
                                  int N1, int N2, int N3, void *stream) {
  clear_error();
  CHECK_PTR(grad_out); CHECK_PTR(weight); CHECK_PTR(grad_image);
  RETURN_IF(check_dims(N1, N2, N3));
  return launch_linear_image_grad(grad_out, weight, grad_image, N1, N2, N3, as_stream(stream));
}

// ---- grid transfer ---------------------------------------------------------------

static int check_grid_dtype(int dt) {
  MLPCG_REQUIRE(dt == MLPCG_F32 || dt == MLPCG_BF16, MLPCG_ERR_UNSUPPORTED,
                "grid transfer dtype must be F32 or BF16");
  return MLPCG_OK;
}

int mlpcg_avg_pool2(const void *x, void *y, int dtype, int B, int N1, int N2, int N3, void *stream) {
  clear_error();
  CHECK_PTR(x); CHECK_PTR(y);
  RETURN_IF(check_grid_dtype(dtype));
  RETURN_IF(check_dims(N1, N2, N3));
  MLPCG_REQUIRE(N1 % 2 == 0 && N2 % 2 == 0 && N3 % 2 == 0, MLPCG_ERR_SHAPE,
                "avg_pool2: sizes must be even (got %d %d %d)", N1, N2, N3);
  MLPCG_REQUIRE(B >= 1 && B <= 65535, MLPCG_ERR_SHAPE, "avg_pool2: bad batch");
  return launch_avg_pool2(x, y, dtype, B, N1, N2, N3, as_stream(stream));
}

int mlpcg_avg_pool2_adjoint(const void *y, void *x, int dtype, int B, int N1, int N2, int N3,
                            void *stream) {
  clear_error();
  CHECK_PTR(x); CHECK_PTR(y);
  RETURN_IF(check_grid_dtype(dtype));
  RETURN_IF(check_dims(N1, N2, N3));
  MLPCG_REQUIRE(N1 % 2 == 0 && N2 % 2 == 0 && N3 % 2 == 0, MLPCG_ERR_SHAPE,
                "avg_pool2_adjoint: sizes must be even");
  MLPCG_REQUIRE(B >= 1 && B <= 65535, MLPCG_ERR_SHAPE, "avg_pool2_adjoint: bad batch");
  return launch_avg_pool2_adjoint(y, x, dtype, B, N1, N2, N3, as_stream(stream));
}

int mlpcg_upsample2(const void *x, void *y, int dtype, int B, int n1, int n2, int n3, void *stream) {
  clear_error();
  CHECK_PTR(x); CHECK_PTR(y);
  RETURN_IF(check_grid_dtype(dtype));
  RETURN_IF(check_dims(n1, n2, n3));
  MLPCG_REQUIRE(B >= 1 && B <= 65535, MLPCG_ERR_SHAPE, "upsample2: bad batch");
  return launch_upsample2(x, y, dtype, B, n1, n2, n3, as_stream(stream));
}

int mlpcg_upsample2_adjoint(const void *y, void *x, int dtype, int B, int n1, int n2, int n3,
                            void *stream) {
  clear_error();
  CHECK_PTR(x); CHECK_PTR(y);
  RETURN_IF(check_grid_dtype(dtype));
  RETURN_IF(check_dims(n1, n2, n3));
  MLPCG_REQUIRE(B >= 1 && B <= 65535, MLPCG_ERR_SHAPE, "upsample2_adjoint: bad batch");
  return launch_upsample2_adjoint(y, x, dtype, B, n1, n2, n3, as_stream(stream));
}

int mlpcg_axpby(const float *c0, const void *x, const float *c1, const void *y, void *out, int dtype,
                int64_t n, void *stream) {
  clear_error();
  CHECK_PTR(c0); CHECK_PTR(x); CHECK_PTR(c1); CHECK_PTR(y); CHECK_PTR(out);
  RETURN_IF(check_grid_dtype(dtype));
  MLPCG_REQUIRE(n >= 0, MLPCG_ERR_ARG, "axpby: negative size");
  if (n == 0) return MLPCG_OK;
  return launch_axpby(c0, x, c1, y, out, dtype, n, as_stream(stream));
}

int mlpcg_laplacian_apply(const uint8_t *flags, const void *x, void *y, int dtype, int N1, int N2, int N3,
                          void *stream) {
  clear_error();
  CHECK_PTR(flags); CHECK_PTR(x); CHECK_PTR(y);
  RETURN_IF(check_dims(N1, N2, N3));
  return launch_laplacian(flags, x, y, dtype, N1, N2, N3, as_stream(stream));
}

int mlpcg_flags_to_image(const uint8_t *flags, float *image, int64_t n, void *stream) {
  clear_error();
  CHECK_PTR(flags); CHECK_PTR(image);
  MLPCG_REQUIRE(n >= 1, MLPCG_ERR_ARG, "flags_to_image: n must be >= 1");
  return launch_flags_to_image(flags, image, n, as_stream(stream));
}

size_t mlpcg_fluid_order_entries(int64_t n) { return n < 1 ? 0 : (size_t)(2 * fluid_blocks(n)); }

int mlpcg_fluid_order(const uint8_t *flags, int64_t n, uint32_t *order, void *stream) {
  clear_error();
  CHECK_PTR(flags); CHECK_PTR(order);
  MLPCG_REQUIRE(n >= 1, MLPCG_ERR_ARG, "fluid_order: n must be >= 1");
  return launch_fluid_order(flags, n, order, as_stream(stream));
}

int mlpcg_scatter_fluid(const double *fluid_values, int64_t m, const uint8_t *flags, const uint32_t *order,
                        int64_t n, double *grid, void *stream) {
  clear_error();
  CHECK_PTR(fluid_values); CHECK_PTR(flags); CHECK_PTR(order); CHECK_PTR(grid);
  MLPCG_REQUIRE(n >= 1 && m >= 0, MLPCG_ERR_ARG, "scatter_fluid: need n >= 1 and m >= 0");
  return launch_scatter_fluid(fluid_values, m, flags, order, n, grid, as_stream(stream));
}

int mlpcg_gather_fluid(const double *grid, const uint8_t *flags, const uint32_t *order, int64_t n,
                       double *fluid_values, int64_t m, void *stream) {
  clear_error();
  CHECK_PTR(grid); CHECK_PTR(flags); CHECK_PTR(order); CHECK_PTR(fluid_values);
  MLPCG_REQUIRE(n >= 1 && m >= 0, MLPCG_ERR_ARG, "gather_fluid: need n >= 1 and m >= 0");
  return launch_gather_fluid(grid, flags, order, n, fluid_values, m, as_stream(stream));
}

int mlpcg_host_mapped(const void *ptr, int *mapped) {
  clear_error();
  CHECK_PTR(ptr); CHECK_PTR(mapped);
  cudaPointerAttributes a{};
  const cudaError_t e = cudaPointerGetAttributes(&a, ptr);
  if (e != cudaSuccess) cudaGetLastError();  // an address CUDA does not know: not mapped
  *mapped = e == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer == ptr ? 1 : 0;
  return MLPCG_OK;
}

size_t mlpcg_dot_workspace(int64_t n) { return dot_workspace(n < 1 ? 1 : n); }

int mlpcg_dot(const void *x, const void *y, int dtype, int64_t n, double *out, void *workspace,
              size_t workspace_bytes, void *stream) {
  clear_error();
  CHECK_PTR(x); CHECK_PTR(y); CHECK_PTR(out); CHECK_PTR(workspace);
  MLPCG_REQUIRE(valid_dtype(dtype), MLPCG_ERR_UNSUPPORTED, "dot: bad dtype %d", dtype);
  MLPCG_REQUIRE(n >= 1, MLPCG_ERR_ARG, "dot: n must be >= 1");
  return launch_dot(x, y, dtype, n, out, workspace, workspace_bytes, as_stream(stream));
}

}  // extern "C"
