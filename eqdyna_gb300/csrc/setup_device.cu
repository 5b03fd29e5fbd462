// Setup on the GPU: the per-element tables and the lumped nodal masses that the reference builds
// on the host before its time loop (assembleGlobalMass, src/assembleGlobalMass.f90:12-38,283-406,
// with calcGlobalShapeFunc src/calcGlobalShapeFunc.f90:1-75 and calcSSPhi4Hrgls :328-374),
// computed from the mesh alone (coordinates, connectivity, element types, materials).
//
// The element math is eqd::geom::element_tables (eqd_geometry.h), the same source the host case
// builder runs; this translation unit is compiled without floating-point contraction
// (--fmad=false), and binary64 add, multiply, divide and square root are correctly rounded on
// both sides, so every table is bit for bit the host's.  The nodal mass of a node is the sum of
// its incident corner masses in the reference's order (element by element, corners in order),
// taken per node from an incidence list in that order, so it is bit for bit too.
//
// Two users: eqd_gpu_element_tables (tables returned to the caller, the reference layout) and
// eqd_gpu_init when the caller passes no tables (built straight into the device layout, so a
// mesh of 10^8 elements needs none of the ~700 bytes per element of host tables).
#include <algorithm>
#include <vector>

#include "eqd_device.cuh"
#include "eqd_geometry.h"
#include "setup_device.h"

namespace eqd {
namespace {

constexpr int kSetupBlock = 128;

__device__ __forceinline__ void corner_coords(const int32_t *__restrict__ conn, const double *__restrict__ coor,
                                              long long e, double xl[3][8]) {
  for (int k = 0; k < 8; ++k) {
    const long long n = conn[8 * e + k] - 1;
    for (int q = 0; q < 3; ++q) xl[q][k] = coor[3 * n + q];
  }
}

// Tables of elements ids[i] (or e0 + i when ids is null), i < n.  Reference layout (element
// major, as eleshp(3, 8, e) ...) when ld == 0, else component-major rows of stride ld
// (shp[q * ld + i]): the device layout of an element group.
__global__ void __launch_bounds__(kSetupBlock)
    element_tables_kernel(long long e0, const int *__restrict__ ids, int n, int nelem,
                          const int32_t *__restrict__ conn, const double *__restrict__ coor,
                          const int32_t *__restrict__ etype, const double *__restrict__ mat, long long ld,
                          double *__restrict__ shp, double *__restrict__ det, double *__restrict__ em,
                          double *__restrict__ ss, double *__restrict__ phi, double detw_scale,
                          int *__restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long e = ids ? (long long)ids[i] : e0 + i;
  if (e < 0) {  // empty slot of a padded group: zero tables
    if (ld) {
      for (int q = 0; q < 24; ++q) shp[q * ld + i] = 0.0;
      for (int q = 0; q < 32; ++q) phi[q * ld + i] = 0.0;
      for (int q = 0; q < 6; ++q) ss[q * ld + i] = 0.0;
      if (em)
        for (int q = 0; q < 8; ++q) em[q * ld + i] = 0.0;
      det[i] = 0.0;
    }
    return;
  }
  double xl[3][8];
  corner_coords(conn, coor, e, xl);
  double m[5];
  for (int k = 0; k < 5; ++k) m[k] = mat[(size_t)k * nelem + e];
  double t_shp[24], t_det = 0.0, t_em[8], t_ss[6], t_phi[32];
  if (!geom::element_tables(xl, etype[e], m, t_shp, t_det, t_em, t_ss, t_phi)) {
    atomicMin(bad, (int)e);
    return;
  }
  if (ld == 0) {
    const long long o = i;
    for (int q = 0; q < 24; ++q) shp[24 * o + q] = t_shp[q];
    for (int q = 0; q < 32; ++q) phi[32 * o + q] = t_phi[q];
    for (int q = 0; q < 6; ++q) ss[6 * o + q] = t_ss[q];
    for (int k = 0; k < 8; ++k) em[8 * o + k] = t_em[k];
    det[o] = t_det;
  } else {
    for (int q = 0; q < 24; ++q) shp[q * ld + i] = t_shp[q];
    for (int q = 0; q < 32; ++q) phi[q * ld + i] = t_phi[q];
    for (int q = 0; q < 6; ++q) ss[q * ld + i] = t_ss[q];
    if (em)
      for (int k = 0; k < 8; ++k) em[k * ld + i] = t_em[k];
    det[i] = t_det * detw_scale;
  }
}

// Corner masses of every element, [8][nelem], from the reference-layout chunk tables.
__global__ void scatter_corner_mass(const double *__restrict__ em_chunk, long long e0, int n, long long nelem,
                                    double *__restrict__ em_all) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 8; ++k) em_all[k * nelem + e0 + i] = em_chunk[8 * (long long)i + k];
}

// Lumped mass of every node: its incident corner masses summed in the reference's order (the
// incidence list of a node is sorted by element, then corner).
__global__ void nodal_mass_kernel(int nnode, const long long *__restrict__ ptr, const int32_t *__restrict__ inc,
                                  const double *__restrict__ em_all, long long nelem, double *__restrict__ mass) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nnode) return;
  double s = 0.0;
  for (long long q = ptr[j]; q < ptr[j + 1]; ++q) {
    const int r = inc[q];  // 8 e + k
    s += em_all[(long long)(r & 7) * nelem + (r >> 3)];
  }
  mass[j] = s;
}

template <class T>
struct DevBuf {
  T *p = nullptr;
  int alloc(size_t n) {
    if (n == 0) return EQD_OK;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return EQD_ERR_OOM;
    }
    return EQD_OK;
  }
  int upload(const T *h, size_t n) {
    const int rc = alloc(n);
    if (rc || n == 0) return rc;
    return cudaMemcpy(p, h, n * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

// Incidence list of every node in the reference's summation order: ptr[nnode + 1], inc[8 nelem]
// entries 8 e + k (element e 0-based, corner k), sorted by e then k.  Built on the host by a
// counting pass and a fill in element order (which sorts each list by itself).
int node_incidences(const eqd_host_arrays &a, std::vector<long long> &ptr, std::vector<int32_t> &inc) {
  const int nn = a.nnode, ne = a.nelem;
  if ((long long)ne * 8 > 0x7fffffffLL) return EQD_ERR_UNSUPPORTED;
  ptr.assign((size_t)nn + 1, 0);
  for (long long q = 0; q < 8 * (long long)ne; ++q) {
    const int n = a.nodeElemIdRelation[q];
    if (n < 1 || n > nn) return EQD_ERR_INPUT;
    ++ptr[n];
  }
  for (int j = 0; j < nn; ++j) ptr[j + 1] += ptr[j];
  inc.resize(8 * (size_t)ne);
  std::vector<long long> fill(ptr.begin(), ptr.end() - 1);
  for (long long q = 0; q < 8 * (long long)ne; ++q) inc[fill[a.nodeElemIdRelation[q] - 1]++] = (int32_t)q;
  return EQD_OK;
}

// Per-element tables of the listed elements straight into a group's device layout (rows of stride
// ld, see element_tables_kernel) from device copies of the mesh; detw = eledet * w.
int device_group_tables(const DeviceMesh &m, const int *d_ids, int n, long long ld, double w, double *shp,
                        double *detw, double *em, double *ss, double *phi, cudaStream_t s) {
  if (n <= 0) return EQD_OK;
  DevBuf<int> bad;
  RC_SETUP(bad.alloc(1));
  const int big = 0x7fffffff;
  EQD_CUDA_OK(cudaMemcpy(bad.p, &big, sizeof(int), cudaMemcpyHostToDevice));
  element_tables_kernel<<<(n + kSetupBlock - 1) / kSetupBlock, kSetupBlock, 0, s>>>(
      0, d_ids, n, m.nelem, m.conn, m.coor, m.etype, m.mat, ld, shp, detw, em, ss, phi, w, bad.p);
  EQD_CUDA_OK(cudaGetLastError());
  int hb = big;
  EQD_CUDA_OK(cudaMemcpy(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
  return hb == big ? EQD_OK : EQD_ERR_INPUT;  // a non-positive determinant
}

// Lumped nodal masses (one per Fortran node) on the device from device copies of the mesh.
int device_nodal_mass(const eqd_host_arrays &a, const DeviceMesh &m, std::vector<double> &mass) {
  std::vector<long long> ptr;
  std::vector<int32_t> inc;
  RC_SETUP(node_incidences(a, ptr, inc));
  const long long ne = a.nelem;
  const int chunk = 1 << 22;
  DevBuf<double> em_all, shp, det, em, ss, phi;
  DevBuf<int> bad;
  RC_SETUP(em_all.alloc(8 * (size_t)ne));
  const int c0 = (int)std::min<long long>(chunk, std::max<long long>(ne, 1));
  RC_SETUP(shp.alloc(24 * (size_t)c0));
  RC_SETUP(det.alloc(c0));
  RC_SETUP(em.alloc(8 * (size_t)c0));
  RC_SETUP(ss.alloc(6 * (size_t)c0));
  RC_SETUP(phi.alloc(32 * (size_t)c0));
  RC_SETUP(bad.alloc(1));
  const int big = 0x7fffffff;
  EQD_CUDA_OK(cudaMemcpy(bad.p, &big, sizeof(int), cudaMemcpyHostToDevice));
  for (long long e0 = 0; e0 < ne; e0 += chunk) {
    const int n = (int)std::min<long long>(chunk, ne - e0);
    const int g = (n + kSetupBlock - 1) / kSetupBlock;
    element_tables_kernel<<<g, kSetupBlock>>>(e0, nullptr, n, a.nelem, m.conn, m.coor, m.etype, m.mat, 0, shp.p,
                                              det.p, em.p, ss.p, phi.p, 1.0, bad.p);
    scatter_corner_mass<<<g, kSetupBlock>>>(em.p, e0, n, ne, em_all.p);
  }
  EQD_CUDA_OK(cudaGetLastError());
  DevBuf<long long> dptr;
  DevBuf<int32_t> dinc;
  DevBuf<double> dmass;
  RC_SETUP(dptr.upload(ptr.data(), ptr.size()));
  RC_SETUP(dinc.upload(inc.data(), inc.size()));
  RC_SETUP(dmass.alloc(a.nnode));
  nodal_mass_kernel<<<(a.nnode + 255) / 256, 256>>>(a.nnode, dptr.p, dinc.p, em_all.p, ne, dmass.p);
  EQD_CUDA_OK(cudaGetLastError());
  mass.resize(a.nnode);
  EQD_CUDA_OK(cudaMemcpy(mass.data(), dmass.p, sizeof(double) * a.nnode, cudaMemcpyDeviceToHost));
  int hb = big;
  EQD_CUDA_OK(cudaMemcpy(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
  return hb == big ? EQD_OK : EQD_ERR_INPUT;
}

int DeviceMesh::upload(const eqd_host_arrays &a) {
  nelem = a.nelem;
  const size_t ne = (size_t)a.nelem, nn = (size_t)a.nnode;
  auto up = [&](auto *&dst, const auto *src, size_t n) -> int {
    using T = std::remove_const_t<std::remove_pointer_t<decltype(src)>>;
    void *p = nullptr;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return EQD_ERR_OOM;
    }
    dst = static_cast<std::remove_reference_t<decltype(dst)>>(p);
    return cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
  };
  RC_SETUP(up(conn, a.nodeElemIdRelation, 8 * ne));
  RC_SETUP(up(coor, a.meshCoor, 3 * nn));
  RC_SETUP(up(etype, a.elemTypeArr, ne));
  RC_SETUP(up(mat, a.mat, 5 * ne));
  return EQD_OK;
}

DeviceMesh::~DeviceMesh() {
  if (conn) cudaFree(conn);
  if (coor) cudaFree(coor);
  if (etype) cudaFree(etype);
  if (mat) cudaFree(mat);
}

}  // namespace eqd

using namespace eqd;

extern "C" int eqd_gpu_element_tables(int32_t device, const eqd_host_arrays *a, double *eleshp, double *eledet,
                                      double *elemass, double *ss, double *phi, double *nodalMassArr,
                                      double *fnms) {
  if (!a || a->nnode <= 0 || a->nelem <= 0 || !a->nodeElemIdRelation || !a->elemTypeArr || !a->meshCoor || !a->mat)
    return EQD_ERR_INPUT;
  if (nodalMassArr && (!a->eqNumIndexArr || !a->eqNumStartIndexLoc || !a->numOfDofPerNodeArr || a->neq <= 0))
    return EQD_ERR_INPUT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return EQD_ERR_NO_DEVICE;
  }
  EQD_CUDA_OK(cudaSetDevice(device));
  for (long long q = 0; q < 8 * (long long)a->nelem; ++q)
    if (a->nodeElemIdRelation[q] < 1 || a->nodeElemIdRelation[q] > a->nnode) return EQD_ERR_INPUT;
  DeviceMesh m;
  RC_SETUP(m.upload(*a));
  const long long ne = a->nelem;
  if (eleshp || eledet || elemass || ss || phi) {
    const int chunk = 1 << 22;
    const int c0 = (int)std::min<long long>(chunk, ne);
    DevBuf<double> d_shp, d_det, d_em, d_ss, d_phi;
    DevBuf<int> bad;
    RC_SETUP(d_shp.alloc(24 * (size_t)c0));
    RC_SETUP(d_det.alloc(c0));
    RC_SETUP(d_em.alloc(8 * (size_t)c0));
    RC_SETUP(d_ss.alloc(6 * (size_t)c0));
    RC_SETUP(d_phi.alloc(32 * (size_t)c0));
    RC_SETUP(bad.alloc(1));
    const int big = 0x7fffffff;
    EQD_CUDA_OK(cudaMemcpy(bad.p, &big, sizeof(int), cudaMemcpyHostToDevice));
    std::vector<double> h_em(8 * (size_t)c0);
    for (long long e0 = 0; e0 < ne; e0 += chunk) {
      const int n = (int)std::min<long long>(chunk, ne - e0);
      element_tables_kernel<<<(n + kSetupBlock - 1) / kSetupBlock, kSetupBlock>>>(
          e0, nullptr, n, a->nelem, m.conn, m.coor, m.etype, m.mat, 0, d_shp.p, d_det.p, d_em.p, d_ss.p, d_phi.p, 1.0,
          bad.p);
      EQD_CUDA_OK(cudaGetLastError());
      if (eleshp) EQD_CUDA_OK(cudaMemcpy(eleshp + 24 * e0, d_shp.p, sizeof(double) * 24 * n, cudaMemcpyDeviceToHost));
      if (eledet) EQD_CUDA_OK(cudaMemcpy(eledet + e0, d_det.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
      if (ss) EQD_CUDA_OK(cudaMemcpy(ss + 6 * e0, d_ss.p, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost));
      if (phi) EQD_CUDA_OK(cudaMemcpy(phi + 32 * e0, d_phi.p, sizeof(double) * 32 * n, cudaMemcpyDeviceToHost));
      if (elemass) {
        EQD_CUDA_OK(cudaMemcpy(h_em.data(), d_em.p, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < n; ++i)
          for (int k = 0; k < 8; ++k)
            for (int q = 0; q < 3; ++q) elemass[24 * (e0 + i) + 3 * k + q] = h_em[8 * i + k];
      }
    }
    int hb = big;
    EQD_CUDA_OK(cudaMemcpy(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (hb != big) return EQD_ERR_INPUT;  // non-positive determinant
  }
  if (nodalMassArr || fnms) {
    std::vector<double> mass;
    RC_SETUP(device_nodal_mass(*a, m, mass));
    if (fnms) std::copy(mass.begin(), mass.end(), fnms);
    if (nodalMassArr) {
      std::fill(nodalMassArr, nodalMassArr + a->neq, 0.0);
      for (int j = 0; j < a->nnode; ++j) {
        const int nd = a->numOfDofPerNodeArr[j];
        for (int k = 0; k < nd; ++k) {
          const int e = a->eqNumIndexArr[a->eqNumStartIndexLoc[j] + k];
          if (e > 0 && e <= a->neq) nodalMassArr[e - 1] = mass[j];
        }
      }
    }
  }
  return EQD_OK;
}
