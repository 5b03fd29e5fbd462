// Learned Newton initial guess: device parameter block management (training kernels follow).
#include "mlp_common.cuh"

namespace eqd {

const void *mlp_device_params(Context &c) { return c.mlp; }

int mlp_init(Context &c) {
  (void)c;
  return EQD_OK;
}

void mlp_free(Context &c) {
  if (c.mlp) cudaFree(c.mlp);
  c.mlp = nullptr;
}

}  // namespace eqd
