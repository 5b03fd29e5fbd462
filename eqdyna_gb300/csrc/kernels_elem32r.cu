// Element kernels of the binary32 form, record-indexed layout.
//
// On EQdyna's structured hexahedral meshes most elements share their geometry and material
// exactly (a uniform grid has one distinct record), so the per-element geometry tables of the
// streamed layout (shape gradients, hourglass vectors and stiffness, det, lambda, mu: ~260 bytes
// per element) are replaced by one 32-bit record index per element into a small table of distinct
// binary32 records that stays in L1/L2.  The PML factors (a_k, b_k) are indexed per axis (16 bits
// each, two 32-bit rows) into a table of the distinct pairs of each axis.  Values are
// bit-identical to the streamed layout's; results differ only through the order of the binary32
// L2 reductions.
//
// A group with a single record (a uniform grid) runs the UNI variant: the record is a kernel
// parameter (__grid_constant__), so its values are constant-bank operands with no load
// instruction, and the PML gather reads the 24 products det * shape gradient from shared memory.
//
// Per tile (CTA of 128 elements): one elected thread bulk-copies the per-element rows that remain
// (stress, record index, PML axis indices, initial stress, pore pressure) and the incidence list
// into shared memory while all threads gather the tile's node data; then the element math and the
// node gather of elem32_common.cuh.
#include <algorithm>
#include <type_traits>
#include <vector>

#include "elem32r_body.cuh"

namespace eqd {

using namespace e32;

namespace {

// One group of one context: arguments in parameter space (record values become constant-bank
// operands in the UNI variant).
template <bool BODY, bool PLASTIC, int HG, bool UNI, bool QM>
__global__ void __launch_bounds__(kTile) elem_interior_rec(const __grid_constant__ ElemArgs32 a) {
  interior_rec_body<BODY, PLASTIC, HG, UNI, QM>(a, blockIdx.x);
}
template <bool BODY, bool S0, int HG, bool UNI>
__global__ void __launch_bounds__(kTile) elem_pml_rec(const __grid_constant__ ElemArgs32 a) {
  pml_rec_body<BODY, S0, HG, UNI>(a, blockIdx.x);
}

// The same group of every member of an ensemble in one launch: each CTA finds its member from the
// tile prefix sums and copies the member's arguments into shared memory.
__device__ __forceinline__ int load_member(const ElemArgs32 *__restrict__ args, const int *__restrict__ start,
                                           int n, ElemArgs32 &a) {
  const int m = elem_batch_member(start, n, blockIdx.x);
  const int *src = reinterpret_cast<const int *>(args + m);
  int *dst = reinterpret_cast<int *>(&a);
  for (int q = threadIdx.x; q < (int)(sizeof(ElemArgs32) / 4); q += blockDim.x) dst[q] = src[q];
  __syncthreads();
  return blockIdx.x - start[m];
}
template <bool BODY, bool PLASTIC, int HG, bool QM>
__global__ void __launch_bounds__(kTile) elem_interior_rec_batched(const ElemArgs32 *__restrict__ args,
                                                                   const int *__restrict__ start, int n) {
  __shared__ __align__(16) ElemArgs32 a;
  const int tile = load_member(args, start, n, a);
  if (a.g.nrec == 1) interior_rec_body<BODY, PLASTIC, HG, true, QM>(a, tile);
  else interior_rec_body<BODY, PLASTIC, HG, false, QM>(a, tile);
}
template <bool BODY, bool S0, int HG>
__global__ void __launch_bounds__(kTile) elem_pml_rec_batched(const ElemArgs32 *__restrict__ args,
                                                              const int *__restrict__ start, int n) {
  __shared__ __align__(16) ElemArgs32 a;
  const int tile = load_member(args, start, n, a);
  if (a.g.nrec == 1) pml_rec_body<BODY, S0, HG, true>(a, tile);
  else pml_rec_body<BODY, S0, HG, false>(a, tile);
}

ElemArgs32 elem_args(const Context &c, bool interior, const ElemConst32 &k) {
  ElemArgs32 a;
  a.g = interior ? c.gi32 : c.gp32;
  a.vel32 = c.vel32;
  a.dl32 = c.dl32;
  a.F = c.F32;
  a.F9 = c.F9_32;
  a.nnode = c.nnode;
  a.n_int = c.n_int;
  a.npml = c.npml;
  a.err = c.d_err;
  a.k = k;
  a.rp = c.rec0[interior ? 0 : 1];
  return a;
}

// Kernel variant of a context's group: template flags (BODY, PLASTIC / S0, HG) as a small code.
struct Variant {
  bool body, plastic, s0;
  int hg;
  bool q;  // Q memory variables (elastic only)
};
Variant variant_of(const Context &c) {
  return Variant{(c.sc.rdampm != 0.0) || (c.sc.C_elastic == 0), c.sc.C_elastic == 0, c.gp32.stress0 != nullptr,
                 c.sc.C_hg == 2 ? 2 : 1, c.sc.C_Q != 0};
}

template <bool BODY, bool PLASTIC, int HG, bool QM>
int launch_interior(Context &c, cudaStream_t s, const ElemConst32 &k) {
  const ElemArgs32 a = elem_args(c, true, k);
  const size_t sm = rec_smem<RecInterior<BODY, PLASTIC, HG, QM>>(a.g.max_tile_nodes);
  if (a.g.nrec == 1) {
    auto kern = elem_interior_rec<BODY, PLASTIC, HG, true, QM>;
    if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
    kern<<<a.g.ntiles, kTile, sm, s>>>(a);
  } else {
    auto kern = elem_interior_rec<BODY, PLASTIC, HG, false, QM>;
    if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
    kern<<<a.g.ntiles, kTile, sm, s>>>(a);
  }
  return EQD_OK;
}

template <bool BODY, bool S0, int HG>
int launch_pml(Context &c, cudaStream_t s, const ElemConst32 &k) {
  const ElemArgs32 a = elem_args(c, false, k);
  if (a.g.nrec == 1) {
    const size_t sm = rec_smem<RecPml<BODY, S0, HG, true>>(a.g.max_tile_nodes);
    auto kern = elem_pml_rec<BODY, S0, HG, true>;
    if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
    kern<<<a.g.ntiles, kTile, sm, s>>>(a);
  } else {
    const size_t sm = rec_smem<RecPml<BODY, S0, HG>>(a.g.max_tile_nodes);
    auto kern = elem_pml_rec<BODY, S0, HG, false>;
    if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
    kern<<<a.g.ntiles, kTile, sm, s>>>(a);
  }
  return EQD_OK;
}

template <int HG>
int launch_hg(Context &c, cudaStream_t s, const ElemConst32 &k, bool interior) {
  const Variant v = variant_of(c);
  if (interior) {
    if (v.plastic && v.q)  // plasticity with Q: C_Q = 2 only (the reference stops on C_Q = 1)
      return v.body ? launch_interior<true, true, HG, true>(c, s, k) : launch_interior<false, true, HG, true>(c, s, k);
    if (v.plastic)
      return v.body ? launch_interior<true, true, HG, false>(c, s, k) : launch_interior<false, true, HG, false>(c, s, k);
    if (v.q)
      return v.body ? launch_interior<true, false, HG, true>(c, s, k) : launch_interior<false, false, HG, true>(c, s, k);
    return v.body ? launch_interior<true, false, HG, false>(c, s, k) : launch_interior<false, false, HG, false>(c, s, k);
  }
  if (v.body) return v.s0 ? launch_pml<true, true, HG>(c, s, k) : launch_pml<true, false, HG>(c, s, k);
  return v.s0 ? launch_pml<false, true, HG>(c, s, k) : launch_pml<false, false, HG>(c, s, k);
}

// ---- ensembles ----------------------------------------------------------------------------------
template <bool BODY, bool PLASTIC, int HG, bool QM>
int launch_interior_batched(const ElemArgs32 *args, const int *start, int n, int tiles, int Mmax, cudaStream_t s) {
  const size_t sm = rec_smem<RecInterior<BODY, PLASTIC, HG, QM>>(Mmax);
  auto kern = elem_interior_rec_batched<BODY, PLASTIC, HG, QM>;
  if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
  kern<<<tiles, kTile, sm, s>>>(args, start, n);
  return EQD_OK;
}
template <bool BODY, bool S0, int HG>
int launch_pml_batched(const ElemArgs32 *args, const int *start, int n, int tiles, int Mmax, cudaStream_t s) {
  const size_t sm = rec_smem<RecPml<BODY, S0, HG>>(Mmax);
  auto kern = elem_pml_rec_batched<BODY, S0, HG>;
  if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
  kern<<<tiles, kTile, sm, s>>>(args, start, n);
  return EQD_OK;
}
template <int HG>
int launch_batched_hg(const Variant &v, bool interior, const ElemArgs32 *args, const int *start, int n, int tiles,
                      int Mmax, cudaStream_t s) {
  if (interior) {
    if (v.plastic && v.q)
      return v.body ? launch_interior_batched<true, true, HG, true>(args, start, n, tiles, Mmax, s)
                    : launch_interior_batched<false, true, HG, true>(args, start, n, tiles, Mmax, s);
    if (v.plastic)
      return v.body ? launch_interior_batched<true, true, HG, false>(args, start, n, tiles, Mmax, s)
                    : launch_interior_batched<false, true, HG, false>(args, start, n, tiles, Mmax, s);
    if (v.q)
      return v.body ? launch_interior_batched<true, false, HG, true>(args, start, n, tiles, Mmax, s)
                    : launch_interior_batched<false, false, HG, true>(args, start, n, tiles, Mmax, s);
    return v.body ? launch_interior_batched<true, false, HG, false>(args, start, n, tiles, Mmax, s)
                  : launch_interior_batched<false, false, HG, false>(args, start, n, tiles, Mmax, s);
  }
  if (v.body)
    return v.s0 ? launch_pml_batched<true, true, HG>(args, start, n, tiles, Mmax, s)
                : launch_pml_batched<true, false, HG>(args, start, n, tiles, Mmax, s);
  return v.s0 ? launch_pml_batched<false, true, HG>(args, start, n, tiles, Mmax, s)
              : launch_pml_batched<false, false, HG>(args, start, n, tiles, Mmax, s);
}

struct ElemBatch {
  int n = 0;
  Variant v{};
  ElemArgs32 *d_args[2] = {nullptr, nullptr};  // interior, PML
  int *d_start[2] = {nullptr, nullptr};         // [n + 1] tile prefix sums
  int tiles[2] = {0, 0}, Mmax[2] = {0, 0};
  std::vector<ElemArgs32> h_args[2];
};

}  // namespace

int record_length(int hg, bool body, bool q) {
  const int n = (hg == 2 ? TabCommon<2>::STR : TabCommon<1>::STR) + (body ? 8 : 0) + (q ? 5 : 0);
  static_assert(TabCommon<1>::STR + 8 + 5 <= kRecMax, "record longer than RecordParam");
  return (n + 3) / 4 * 4;
}

int launch_elements_rec(Context &c, cudaStream_t s, const ElemConst32 &k, bool interior) {
  return c.sc.C_hg == 2 ? launch_hg<2>(c, s, k, interior) : launch_hg<1>(c, s, k, interior);
}

// Builds (or refreshes) the element tables of an ensemble.  Every member must run the binary32
// form with record-indexed tables and the same kernel variant.
int elem_batch_update(void **handle, Context *const *m, int n, const ElemConst *kd) {
  if (n <= 0) return EQD_ERR_INPUT;
  ElemBatch *b = static_cast<ElemBatch *>(*handle);
  const Variant v = variant_of(*m[0]);
  for (int i = 0; i < n; ++i) {
    const Variant w = variant_of(*m[i]);
    if (!m[i]->fp32 || w.body != v.body || w.plastic != v.plastic || w.s0 != v.s0 || w.hg != v.hg || w.q != v.q)
      return EQD_ERR_UNSUPPORTED;
    for (int grp = 0; grp < 2; ++grp) {
      const ElemGroup<float> &g = grp == 0 ? m[i]->gi32 : m[i]->gp32;
      if (g.ne > 0 && g.nrec == 0) return EQD_ERR_UNSUPPORTED;  // streamed tables
    }
  }
  if (!b) {
    b = new ElemBatch();
    b->n = n;
    b->v = v;
    for (int grp = 0; grp < 2; ++grp) {
      std::vector<int> start(n + 1, 0);
      for (int i = 0; i < n; ++i) {
        const ElemGroup<float> &g = grp == 0 ? m[i]->gi32 : m[i]->gp32;
        start[i + 1] = start[i] + (g.ne > 0 ? g.ntiles : 0);
        b->Mmax[grp] = std::max(b->Mmax[grp], g.max_tile_nodes);
      }
      b->tiles[grp] = start[n];
      if (cudaMalloc(&b->d_start[grp], sizeof(int) * (n + 1)) != cudaSuccess ||
          cudaMalloc(&b->d_args[grp], sizeof(ElemArgs32) * n) != cudaSuccess) {
        elem_batch_free(b);
        return EQD_ERR_OOM;
      }
      cudaMemcpy(b->d_start[grp], start.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice);
      b->h_args[grp].resize(n);
    }
    *handle = b;
  }
  if (b->n != n) return EQD_ERR_INPUT;
  for (int grp = 0; grp < 2; ++grp) {
    for (int i = 0; i < n; ++i) {
      const ElemConst &q = kd[i];
      const ElemConst32 k{(float)q.dt, (float)q.rdampk, (float)q.rdampm, (float)q.gz,
                          (float)q.ccosphi, (float)q.sinphi, (float)q.relax};
      b->h_args[grp][i] = elem_args(*m[i], grp == 0, k);
    }
    EQD_CUDA_OK(cudaMemcpy(b->d_args[grp], b->h_args[grp].data(), sizeof(ElemArgs32) * n, cudaMemcpyHostToDevice));
  }
  return EQD_OK;
}

int elem_batch_tables(const void *handle, const void *args[2], const int *start[2], int tiles[2], int Mmax[2],
                      int variant[5]) {
  const ElemBatch *b = static_cast<const ElemBatch *>(handle);
  if (!b) return EQD_ERR_STATE;
  for (int grp = 0; grp < 2; ++grp) {
    args[grp] = b->d_args[grp];
    start[grp] = b->d_start[grp];
    tiles[grp] = b->tiles[grp];
    Mmax[grp] = b->Mmax[grp];
  }
  variant[0] = b->v.body;
  variant[1] = b->v.plastic;
  variant[2] = b->v.s0;
  variant[3] = b->v.hg;
  variant[4] = b->v.q;
  return EQD_OK;
}

int launch_elements_batched(const void *handle, cudaStream_t s, int part) {
  const ElemBatch *b = static_cast<const ElemBatch *>(handle);
  for (int grp = 0; grp < 2; ++grp) {
    if ((grp == 0 && part == 1) || (grp == 1 && part == 0) || b->tiles[grp] == 0) continue;
    const int rc = b->v.hg == 2
                       ? launch_batched_hg<2>(b->v, grp == 0, b->d_args[grp], b->d_start[grp], b->n, b->tiles[grp],
                                              b->Mmax[grp], s)
                       : launch_batched_hg<1>(b->v, grp == 0, b->d_args[grp], b->d_start[grp], b->n, b->tiles[grp],
                                              b->Mmax[grp], s);
    if (rc) return rc;
  }
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

void elem_batch_free(void *handle) {
  ElemBatch *b = static_cast<ElemBatch *>(handle);
  if (!b) return;
  for (int grp = 0; grp < 2; ++grp) {
    if (b->d_args[grp]) cudaFree(b->d_args[grp]);
    if (b->d_start[grp]) cudaFree(b->d_start[grp]);
  }
  delete b;
}

}  // namespace eqd
