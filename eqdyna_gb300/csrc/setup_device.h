// Setup on the GPU (setup_device.cu): per-element tables and nodal masses from the mesh alone.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "eqdyna_gb300.h"

namespace eqd {

#define RC_SETUP(x)           \
  do {                        \
    int rc_ = (x);            \
    if (rc_) return rc_;      \
  } while (0)

// Device copies of the mesh arrays the tables are computed from (Fortran layout and numbering).
struct DeviceMesh {
  int nelem = 0;
  int32_t *conn = nullptr;   // nodeElemIdRelation (8, nelem), 1-based node ids
  double *coor = nullptr;    // meshCoor (3, nnode)
  int32_t *etype = nullptr;  // elemTypeArr (nelem)
  double *mat = nullptr;     // mat (nelem, 5)
  int upload(const eqd_host_arrays &a);
  DeviceMesh() = default;
  DeviceMesh(const DeviceMesh &) = delete;
  DeviceMesh &operator=(const DeviceMesh &) = delete;
  ~DeviceMesh();
};

// Incidences of every node in the reference's summation order (element, then corner).
int node_incidences(const eqd_host_arrays &a, std::vector<long long> &ptr, std::vector<int32_t> &inc);

// Tables of the n elements d_ids[i] (0-based Fortran element numbers, -1 for an empty slot) into
// component-major device rows of stride ld: shp[24], phi[32], ss[6], em[8] (em may be null) and
// detw = eledet * w.  EQD_ERR_INPUT for a non-positive determinant.
int device_group_tables(const DeviceMesh &m, const int *d_ids, int n, long long ld, double w, double *shp,
                        double *detw, double *em, double *ss, double *phi, cudaStream_t s);

// Lumped mass of every Fortran node (the value of each of its equations in nodalMassArr, and fnms).
int device_nodal_mass(const eqd_host_arrays &a, const DeviceMesh &m, std::vector<double> &mass);

}  // namespace eqd
