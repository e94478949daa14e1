// Library-wide entry points: status words, version, solve defaults.
#include "arap_common.cuh"

namespace arap {

int status_read_clear(int* status_dev, cudaStream_t s) {
  int v = 0;
  if (cudaMemcpyAsync(&v, status_dev, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemsetAsync(status_dev, 0, sizeof(int), s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  return v;
}

}  // namespace arap

extern "C" int arap_status_read(int32_t* status_dev, arap_stream_t stream) {
  if (!status_dev) return ARAP_EBADINPUT;
  return arap::status_read_clear(status_dev, (cudaStream_t)stream);
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
  cfg->spin_limit = 0;
  cfg->coarse_reuse = 0.0f;
}
