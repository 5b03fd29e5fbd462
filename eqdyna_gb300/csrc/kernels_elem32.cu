// Element kernels of the binary32 form.
#include "eqd_device.cuh"

namespace eqd {

int launch_elements_f32(Context &c, cudaStream_t s, const ElemConst &k, int part) {
  (void)c; (void)s; (void)k; (void)part;
  return EQD_ERR_UNSUPPORTED;
}

}  // namespace eqd

namespace eqd {
int upload_fp32_tables(Context &c) {
  (void)c;
  return EQD_ERR_UNSUPPORTED;
}
}  // namespace eqd
