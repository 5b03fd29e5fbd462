// Element internal-force pass that allocates no device memory (eqd_gpu_elem_forces_noalloc).
//
// For callers that cannot call cudaMalloc — a Fortran code whose globalvar arrays already live on
// the device under OpenACC or CUDA Fortran data management, or a host program that plans all
// device memory up front and forbids allocation during the run — this entry point runs the
// interior element pass directly on the caller's device-resident Fortran arrays.  Its only
// scratch, the per-node force accumulator, is a file-scope static device array with a fixed
// capacity of kNoallocMaxNodes nodes (3 x 524,288 doubles = 12 MiB), which every GPU that loads
// the library holds until the process exits.
//
// The math is that of the interior element kernel of the time step (one-point hexahedron or
// degenerated wedge, elastic Hooke update, Kosloff-Frazier stiffness hourglass); it reads the
// Fortran layout (element-major tables) instead of the step's structure-of-arrays layout.
//
// The tables are on the device, where the host cannot look at them before the launch, so the
// kernel checks every element's node ids (1 .. nnode) and stress offset (0 .. size_stress - 6)
// itself: an element that fails is skipped (no stress update, no force) and counted in a second
// file-scope device word, which the call reads back once its work is done.
#include <mutex>

#include "eqd_device.cuh"

namespace eqd {
namespace {

constexpr int kNoallocMaxNodes = 1 << 19;
constexpr int kNoallocBlock = 128;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_force[3 * kNoallocMaxNodes];
// elements skipped by the last call because of an out-of-range node id or stress offset
static __device__ int g_noalloc_bad;

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[kMaxDevices] = {nullptr};

__global__ void noalloc_clear(double *acc, int n) {
  if (blockIdx.x == 0 && threadIdx.x == 0) g_noalloc_bad = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc[i] = 0.0;
}

__global__ void __launch_bounds__(kNoallocBlock)
    noalloc_elem(eqd_elem_device_view v, double *acc) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= v.nelem) return;
  const int et = v.elemTypeArr[e];
  if (!(et == 1 || et > 10)) return;
  const int nn = v.nnode;
  int n[8];
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    n[a] = v.nodeElemIdRelation[8 * (size_t)e + a] - 1;
    ok = ok && n[a] >= 0 && n[a] < nn;
  }
  const long long so = v.stressCompIndexArr[e];
  ok = ok && so >= 0 && so + 6 <= v.size_stress;
  if (!ok) {  // skipped: contributes nothing, counted for the call to report
    atomicAdd(&g_noalloc_bad, 1);
    return;
  }
  const double *shp = v.eleshp + 24 * (size_t)e;
  const double *phi = v.phi + 32 * (size_t)e;
  double sr[6] = {0, 0, 0, 0, 0, 0};
  double ph[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double bx = shp[3 * a], by = shp[3 * a + 1], bz = shp[3 * a + 2];
    const double *vv = v.velArr + 3 * (size_t)n[a];
    const double *dd = v.dispArr + 3 * (size_t)n[a];
    const double vx = vv[0], vy = vv[1], vz = vv[2];
    sr[0] = fma(bx, vx, sr[0]);
    sr[1] = fma(by, vy, sr[1]);
    sr[2] = fma(bz, vz, sr[2]);
    sr[3] = fma(by, vz, fma(bz, vy, sr[3]));
    sr[4] = fma(bx, vz, fma(bz, vx, sr[4]));
    sr[5] = fma(bx, vy, fma(by, vx, sr[5]));
    const double lx = fma(v.rdampk, vx, dd[0]), ly = fma(v.rdampk, vy, dd[1]), lz = fma(v.rdampk, vz, dd[2]);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const double p = phi[8 * m + a];
      ph[m][0] = fma(p, lx, ph[m][0]);
      ph[m][1] = fma(p, ly, ph[m][1]);
      ph[m][2] = fma(p, lz, ph[m][2]);
    }
  }
  const double lam = v.mat[3 * (size_t)v.nelem + e], mu = v.mat[4 * (size_t)v.nelem + e];
  const double cd = lam + 2.0 * mu;
  const double srate[6] = {cd * sr[0] + lam * sr[1] + lam * sr[2], lam * sr[0] + cd * sr[1] + lam * sr[2],
                           lam * sr[0] + lam * sr[1] + cd * sr[2], mu * sr[3], mu * sr[4], mu * sr[5]};
  double *st = v.stressArr + so;
  const double tw = -v.eledet[e] * v.w;
  double s6[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const double s = fma(srate[i], v.dt, st[i]);
    st[i] = s;
    s6[i] = tw * fma(v.rdampk, srate[i], s);
  }
  const double *ss = v.ss + 6 * (size_t)e;
  double h[4][3];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    h[m][0] = ss[0] * ph[m][0] + ss[1] * ph[m][1] + ss[2] * ph[m][2];
    h[m][1] = ss[1] * ph[m][0] + ss[3] * ph[m][1] + ss[4] * ph[m][2];
    h[m][2] = ss[2] * ph[m][0] + ss[4] * ph[m][1] + ss[5] * ph[m][2];
  }
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double bx = shp[3 * a], by = shp[3 * a + 1], bz = shp[3 * a + 2];
    double f[3] = {bx * s6[0] + bz * s6[4] + by * s6[5], by * s6[1] + bz * s6[3] + bx * s6[5],
                   bz * s6[2] + by * s6[3] + bx * s6[4]};
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const double p = phi[8 * m + a];
      f[0] = fma(-p, h[m][0], f[0]);
      f[1] = fma(-p, h[m][1], f[1]);
      f[2] = fma(-p, h[m][2], f[2]);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) atomicAdd(acc + (size_t)c * nn + n[a], f[c]);
  }
}

__global__ void noalloc_store(const double *acc, double *out, int nn) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x)
#pragma unroll
    for (int c = 0; c < 3; ++c) out[3 * (size_t)i + c] = acc[(size_t)c * nn + i];
}

// Device address of the static accumulator on the current device, looked up once per device.
int scratch_for_current_device(double **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return EQD_ERR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_force) != cudaSuccess || !p) {
      cudaGetLastError();
      return EQD_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_noalloc_ptr[dev];
  return EQD_OK;
}

}  // namespace
}  // namespace eqd

extern "C" int eqd_gpu_elem_forces_noalloc(const eqd_elem_device_view *v, double *force_out, void *stream) {
  using namespace eqd;
  if (!v || !force_out) return EQD_ERR_INPUT;
  if (v->nnode <= 0 || v->nelem < 0 || v->size_stress < 0) return EQD_ERR_INPUT;
  if (v->nnode > kNoallocMaxNodes) return EQD_ERR_INPUT;  // beyond the fixed scratch capacity
  if (!v->nodeElemIdRelation || !v->elemTypeArr || !v->eleshp || !v->eledet || !v->mat || !v->ss ||
      !v->phi || !v->stressArr || !v->stressCompIndexArr || !v->velArr || !v->dispArr)
    return EQD_ERR_INPUT;
  // the pass is the elastic, stiffness-hourglass form only (src/calcElemKU.f90 with C_elastic = 1,
  // C_Q = 0; src/hrglss.f90 with C_hg = 1)
  if (v->C_elastic != 1 || v->C_Q != 0 || v->C_hg != 1) return EQD_ERR_UNSUPPORTED;
  // an error the caller left pending belongs to the caller: report it, keep it, launch nothing
  if (cudaPeekAtLastError() != cudaSuccess) return EQD_ERR_CUDA;
  double *acc = nullptr;
  int rc = scratch_for_current_device(&acc);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int n3 = 3 * v->nnode;
  noalloc_clear<<<(n3 + 255) / 256, 256, 0, s>>>(acc, n3);
  if (cudaGetLastError() != cudaSuccess) return EQD_ERR_CUDA;
  if (v->nelem > 0) {
    noalloc_elem<<<(v->nelem + kNoallocBlock - 1) / kNoallocBlock, kNoallocBlock, 0, s>>>(*v, acc);
    if (cudaGetLastError() != cudaSuccess) return EQD_ERR_CUDA;
  }
  noalloc_store<<<(v->nnode + 255) / 256, 256, 0, s>>>(acc, force_out, v->nnode);
  if (cudaGetLastError() != cudaSuccess) return EQD_ERR_CUDA;
  // wait for this call's work and read the count of skipped elements
  int bad = 0;
  if (cudaMemcpyFromSymbolAsync(&bad, g_noalloc_bad, sizeof(int), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return EQD_ERR_CUDA;
  return bad ? EQD_ERR_INPUT : EQD_OK;
}
