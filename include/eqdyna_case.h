/*
 * eqdyna_case — host-side case setup of eqdyna_gb300.
 *
 * In a deployment the Fortran EQdyna program builds the mesh and the per-element tables
 * (src/eqdyna3d.f90:33-70: readglobal ... meshgen, netcdf_read_on_fault_eqdyna,
 * assembleGlobalMass, init_vel) and hands the resulting globalvar arrays to eqd_gpu_init.
 * This library restates that setup in C++ so that the GPU path can be driven without a Fortran
 * toolchain: it reads the same case directory (bGlobal.txt, bModelGeometry.txt,
 * bFaultGeometry.txt, bMaterial.txt, bStations.txt, [bFault_Rough_Geometry.txt]) plus
 *   on_fault_vars_input.bin  — the 24 fields of on_fault_vars_input.nc as raw little-endian
 *                              binary64, header int32[3] = {24, nfx, nfz}, then the data in
 *                              Fortran order (nfx, nfz, 24) (src/netcdf_io.f90:30-70);
 *   bGPU.txt (optional)      — `key value` lines for switches that are compile-time constants in
 *                              the reference (nPML, R, C_Q, C_hg, kapa_hg, rdampm); absent keys keep
 *                              the reference values (src/globalvar.f90:16-75).
 * The arrays it produces are exactly the Fortran ones (same numbering, same layout).
 */
#ifndef EQDYNA_CASE_H
#define EQDYNA_CASE_H

#include <stdint.h>
#include "eqdyna_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct eqd_case eqd_case;

/* Builds the case found in directory `dir`.  On failure returns a non-zero eqd_status and
 * writes a message retrievable with eqd_case_last_error(). */
int eqd_case_build(const char *dir, eqd_case **out);

/* eqd_case_build with options: flags = EQD_CASE_MESH_ONLY builds the mesh, materials, fault and
 * stations but not the per-element tables or nodal masses (eleshp, eledet, elemass, ss, phi,
 * nodalMassArr and fnms are NULL in the view; about 700 bytes per element less host memory), for
 * eqd_gpu_init to build them on the device. */
#define EQD_CASE_MESH_ONLY 1
int eqd_case_build_opt(const char *dir, int32_t flags, eqd_case **out);

/* Views into the case's arrays (owned by the case; valid until eqd_case_free). */
int eqd_case_view(eqd_case *c, eqd_scalars *s, eqd_host_arrays *a);

/* Length (number of elements) and element size in bytes of a named array of
 * eqd_host_arrays, e.g. "fric", "nodeElemIdRelation".  Returns 0 length for unknown names. */
int64_t eqd_case_array_len(eqd_case *c, const char *name, int32_t *elem_bytes);

/* Derived sizes: nx, ny, nz node lines, number of physical (non-PML) elements, nstep. */
int eqd_case_dims(eqd_case *c, int32_t *nx, int32_t *ny, int32_t *nz, int64_t *n_phys_elem,
                  int32_t *nstep);

/* Grid-line coordinates (x, y, z node lines) of the structured grid. */
int eqd_case_lines(eqd_case *c, const double **x, const double **y, const double **z);

/* Wall seconds of the build's phases: input files, mesh generation, on-fault fields, element
 * tables, mass assembly and finishing. */
int eqd_case_phase_seconds(eqd_case *c, double out[5]);

void eqd_case_free(eqd_case *c);
const char *eqd_case_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* EQDYNA_CASE_H */
