// Library-wide entry points: device status word, version, solve defaults.
#include "arap_common.cuh"

namespace arap {
__device__ int g_status = 0;
}

extern "C" int arap_get_device_status(arap_stream_t stream) {
  int v = 0;
  const int zero = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyFromSymbolAsync(&v, arap::g_status, sizeof(int), 0, cudaMemcpyDeviceToHost, s) !=
      cudaSuccess)
    return ARAP_ECUDA;
  if (cudaMemcpyToSymbolAsync(arap::g_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s) !=
      cudaSuccess)
    return ARAP_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return ARAP_ECUDA;
  return v;
}

extern "C" const char* arap_version(void) { return "arap_gb300 0.1 (sm_103a)"; }

extern "C" void arap_solve_config_default(arap_solve_config* cfg) {
  if (!cfg) return;
  cfg->w_rot = 1.0f;
  cfg->w_reg = 10.0f;
  cfg->w_con = 100.0f;
  cfg->weighting_factor = 1.0f;
  cfg->cons_on_center = 0;
  cfg->max_iters = 30;
  cfg->early_exit = 1;
  cfg->precision = ARAP_PRECISION_PLAIN;
  cfg->pcg_tol = 0.0f;
  cfg->pcg_max_iters = 0;
  cfg->coarse_nodes = 0;
}
