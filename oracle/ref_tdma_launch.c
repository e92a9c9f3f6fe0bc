/* Test infrastructure, not product code: launches the reference's own CUDA
 * TDMA kernel (TridiagKernel<float|double> of
 * veros/core/special/cuda_tdma_kernels.cu:19-63), compiled from that source
 * for sm_103a into a cubin by oracle/ref_tdma.py, with the reference
 * launcher's configuration (CudaTridiag, cuda_tdma_kernels.cu:81-101):
 * 128 threads per block, min(1024, ceil(num_systems / 128)) blocks, the
 * workspace buffer as c' and the output as d'. The kernel is found in the
 * loaded module by its name (the module's function list), so no mangled name
 * is spelled here. Errors are returned as codes, never exit().
 *
 * Used only by the tests and by bench.py's reference arm. */
#include <cuda.h>
#include <string.h>

static CUmodule g_module = 0;
static CUfunction g_kernel[2] = {0, 0}; /* [0] float, [1] double */

/* 0 ok; 1 no context; 2 load failed; 3 kernels not found */
int ref_tdma_load(const char *cubin_path) {
  CUcontext ctx = 0;
  if (cuCtxGetCurrent(&ctx) != CUDA_SUCCESS || !ctx) return 1;
  if (g_module) return (g_kernel[0] && g_kernel[1]) ? 0 : 3;
  if (cuModuleLoad(&g_module, cubin_path) != CUDA_SUCCESS) {
    g_module = 0;
    return 2;
  }
  unsigned int n = 0;
  if (cuModuleGetFunctionCount(&n, g_module) != CUDA_SUCCESS || n == 0 || n > 64) return 3;
  CUfunction fns[64];
  if (cuModuleEnumerateFunctions(fns, n, g_module) != CUDA_SUCCESS) return 3;
  for (unsigned int i = 0; i < n; ++i) {
    const char *name = 0;
    if (cuFuncGetName(&name, fns[i]) != CUDA_SUCCESS || !name) continue;
    if (!strstr(name, "TridiagKernel")) continue;
    if (strstr(name, "TridiagKernelIfE")) g_kernel[0] = fns[i];
    if (strstr(name, "TridiagKernelIdE")) g_kernel[1] = fns[i];
  }
  return (g_kernel[0] && g_kernel[1]) ? 0 : 3;
}

/* buffers = {a, b, c, d, out, workspace} as in the XLA custom call;
 * is_double selects the instantiation. 0 ok; 4 not loaded; 5 launch failed. */
int ref_tdma_launch(void *stream, void **buffers, int num_systems, int system_depth, int is_double) {
  CUfunction f = g_kernel[is_double ? 1 : 0];
  if (!f) return 4;
  const unsigned int block = 128;
  unsigned int grid = (unsigned int)((num_systems + (int)block - 1) / (int)block);
  if (grid > 1024) grid = 1024;
  void *a = buffers[0], *b = buffers[1], *c = buffers[2], *d = buffers[3];
  void *out = buffers[4], *ws = buffers[5];
  void *params[] = {&a, &b, &c, &d, &ws, &out, &num_systems, &system_depth};
  if (cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, (CUstream)stream, params, 0) != CUDA_SUCCESS) return 5;
  return 0;
}
