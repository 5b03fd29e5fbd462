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
#include "elem32_common.cuh"

namespace eqd {

using namespace e32;

namespace {

template <bool BODY, bool PLASTIC, int HG>
struct RecInterior {
  static constexpr int REM = TabCommon<HG>::STR;         // record: 8 corner masses after mu
  static constexpr int STR = 0;                          // shared-memory rows: 6 stress
  static constexpr int POR = 6;                          // 1 pore pressure
  static constexpr int RID = POR + (PLASTIC ? 1 : 0);    // record index (u32)
  static constexpr int N = RID + 1;                      // rows copied
  static constexpr int FS = N;                           // 24 rows of per-corner forces
  static constexpr int NS = N + 24;
};
template <bool BODY, bool S0, int HG>
struct RecPml {
  static constexpr int REM = TabCommon<HG>::STR;
  static constexpr int STR = 0;                          // 15 split-field stress
  static constexpr int ST0 = 15;                         // 6 initial stress
  static constexpr int RID = ST0 + (S0 ? 6 : 0);
  static constexpr int ABID = RID + 1;                   // 2 rows of PML axis indices (u32)
  static constexpr int N = ABID + 2;
  static constexpr int FS = N;
  static constexpr int ES = STR;                         // 6 split-stress sums over the stress rows
  static constexpr int NS = N + 24;
};

template <class L>
struct RecSrc {
  const float *rec;   // this element's record (global, read-only)
  const float *tab;   // per-element rows in shared memory
  int col;
  const float *abt;   // PML: [3][stride][2] (a, b) per axis
  int stride;
  unsigned ab01, ab2; // axis indices: x | y << 16, z
  __device__ float g(int row) const { return __ldg(rec + row); }
  __device__ float em(int a) const { return __ldg(rec + L::REM + a); }
  __device__ float str(int i) const { return tab[(L::STR + i) * kTile + col]; }
  __device__ float por() const { return tab[L::POR * kTile + col]; }
  __device__ float st0(int i) const { return tab[(L::ST0 + i) * kTile + col]; }
  __device__ int ab_index(int k) const {
    return k * stride + (int)(k == 0 ? (ab01 & 0xFFFFu) : (k == 1 ? (ab01 >> 16) : ab2));
  }
  __device__ float pa(int k) const { return __ldg(abt + 2 * ab_index(k)); }
  __device__ float pb(int k) const { return __ldg(abt + 2 * ab_index(k) + 1); }
};

// Table source of a group with one record, held in the kernel's parameter space.
template <class L>
struct UniSrc {
  const RecordParam &r;
  const float *tab;
  int col;
  const float *abt;
  int stride;
  unsigned ab01, ab2;
  __device__ float g(int row) const { return r.v[row]; }
  __device__ float em(int a) const { return r.v[L::REM + a]; }
  __device__ float str(int i) const { return tab[(L::STR + i) * kTile + col]; }
  __device__ float por() const { return tab[L::POR * kTile + col]; }
  __device__ float st0(int i) const { return tab[(L::ST0 + i) * kTile + col]; }
  __device__ int ab_index(int k) const {
    return k * stride + (int)(k == 0 ? (ab01 & 0xFFFFu) : (k == 1 ? (ab01 >> 16) : ab2));
  }
  __device__ float pa(int k) const { return __ldg(abt + 2 * ab_index(k)); }
  __device__ float pb(int k) const { return __ldg(abt + 2 * ab_index(k) + 1); }
};

__device__ __forceinline__ unsigned row_u32(const float *tab, int row, int col) {
  return reinterpret_cast<const unsigned *>(tab)[row * kTile + col];
}

template <bool BODY, bool PLASTIC, int HG, bool UNI>
__global__ void __launch_bounds__(kTile)
    elem_interior_rec(ElemGroup<float> g, const float *__restrict__ vel32, const float *__restrict__ dl32,
                      float *__restrict__ F, int nnode, ElemConst32 k, int *__restrict__ err,
                      const __grid_constant__ RecordParam rp) {
  using L = RecInterior<BODY, PLASTIC, HG>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar;
  const int Mmax = g.max_tile_nodes;
  float *tab = reinterpret_cast<float *>(smem);
  unsigned short *sinc = reinterpret_cast<unsigned short *>(tab + L::NS * kTile);
  unsigned short *slot_of = sinc + 8 * kTile;
  float *sv = reinterpret_cast<float *>(slot_of + 8 * kTile);
  float *sd = sv + 3 * Mmax;
  const int tid = threadIdx.x;
  const int e0 = blockIdx.x * kTile;
  const int ld = g.ld;
  if (tid == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, (unsigned)(L::N * kTile * 4 + 8 * kTile * 2));
    bulk_g2s(sinc, g.tile_inc + (size_t)blockIdx.x * kTile * 8, 8 * kTile * 2, &bar);
    copy_rows(tab, L::STR, g.stress, 6, ld, e0, &bar);
    if (PLASTIC) copy_rows(tab, L::POR, g.porep, 1, ld, e0, &bar);
    copy_rows(tab, L::RID, g.rec_id, 1, ld, e0, &bar);
  }
  __syncthreads();
  int nb;
  const int M = stage_nodes(g, vel32, dl32, nnode, Mmax, sv, sd, nb);
  const bool ok = mbar_wait_bounded(&bar, err);
  const unsigned short *incp = g.tile_incp + g.tile_incp_off[blockIdx.x];
  if (ok) build_slots(incp, M, sinc, slot_of);
  if (__syncthreads_or(!ok)) return;
  const int e = e0 + tid;
  float *fs = tab + L::FS * kTile;
  if (e < g.ne) {
    double *ps = PLASTIC ? g.pstrain + e : nullptr;
    if (UNI) {
      const UniSrc<L> S{rp, tab, tid, nullptr, 0, 0u, 0u};
      interior_element<BODY, PLASTIC, HG>(S, sv, sd, Mmax, slot_of, tid, k, ps, g.stress + e, (size_t)ld, fs);
    } else {
      const RecSrc<L> S{g.rec + (size_t)row_u32(tab, L::RID, tid) * g.rec_len, tab, tid, nullptr, 0, 0u, 0u};
      interior_element<BODY, PLASTIC, HG>(S, sv, sd, Mmax, slot_of, tid, k, ps, g.stress + e, (size_t)ld, fs);
    }
  }
  __syncthreads();
  interior_gather(g, M, nb, incp, sinc, fs, F, nnode);
}

template <bool BODY, bool S0, int HG, bool UNI>
__global__ void __launch_bounds__(kTile)
    elem_pml_rec(ElemGroup<float> g, const float *__restrict__ vel32, const float *__restrict__ dl32,
                 float *__restrict__ F, float *__restrict__ F9, int nnode, int n_int, int npml,
                 ElemConst32 k, int *__restrict__ err, const __grid_constant__ RecordParam rp) {
  using L = RecPml<BODY, S0, HG>;
  using C = TabCommon<HG>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ float cw[24];  // UNI: det * shape gradient (3 a + k) of the group's record
  const int Mmax = g.max_tile_nodes;
  float *tab = reinterpret_cast<float *>(smem);
  unsigned short *sinc = reinterpret_cast<unsigned short *>(tab + L::NS * kTile);
  unsigned short *slot_of = sinc + 8 * kTile;
  float *sv = reinterpret_cast<float *>(slot_of + 8 * kTile);
  float *sd = sv + 3 * Mmax;
  const int tid = threadIdx.x;
  const int e0 = blockIdx.x * kTile;
  const int ld = g.ld;
  if (tid == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, (unsigned)(L::N * kTile * 4 + 8 * kTile * 2));
    bulk_g2s(sinc, g.tile_inc + (size_t)blockIdx.x * kTile * 8, 8 * kTile * 2, &bar);
    copy_rows(tab, L::STR, g.stress, 15, ld, e0, &bar);
    if (S0) copy_rows(tab, L::ST0, g.stress0, 6, ld, e0, &bar);
    copy_rows(tab, L::RID, g.rec_id, 1, ld, e0, &bar);
    copy_rows(tab, L::ABID, g.ab_id, 2, ld, e0, &bar);
  }
  if (UNI && tid < 24) cw[tid] = rp.v[C::DET] * rp.v[C::SHP + tid];
  __syncthreads();
  int nb;
  const int M = stage_nodes(g, vel32, dl32, nnode, Mmax, sv, sd, nb);
  const bool ok = mbar_wait_bounded(&bar, err);
  const unsigned short *incp = g.tile_incp + g.tile_incp_off[blockIdx.x];
  if (ok) build_slots(incp, M, sinc, slot_of);
  if (__syncthreads_or(!ok)) return;
  const int e = e0 + tid;
  float *cfh = tab + L::FS * kTile;
  float *es = tab + L::ES * kTile;
  const float *rec = g.rec;
  const int rlen = g.rec_len;
  if (e < g.ne) {
    const unsigned ab01 = row_u32(tab, L::ABID, tid), ab2 = row_u32(tab, L::ABID + 1, tid);
    if (UNI) {
      const UniSrc<L> S{rp, tab, tid, g.ab_tab, g.ab_stride, ab01, ab2};
      pml_element<BODY, S0, HG>(S, sv, sd, Mmax, slot_of, tid, k, g.stress + e, (size_t)ld, es, cfh);
    } else {
      const RecSrc<L> S{rec + (size_t)row_u32(tab, L::RID, tid) * rlen, tab, tid, g.ab_tab, g.ab_stride,
                        ab01, ab2};
      pml_element<BODY, S0, HG>(S, sv, sd, Mmax, slot_of, tid, k, g.stress + e, (size_t)ld, es, cfh);
    }
  }
  __syncthreads();
  if (UNI) {
    auto w_of = [&](int, int a, float &wx, float &wy, float &wz) {
      wx = cw[3 * a];
      wy = cw[3 * a + 1];
      wz = cw[3 * a + 2];
    };
    pml_gather(g, M, nb, incp, sinc, es, cfh, w_of, F, F9, nnode, n_int, npml);
  } else {
    auto src_of = [&](int el) {
      return RecSrc<L>{rec + (size_t)row_u32(tab, L::RID, el) * rlen, tab, el, nullptr, 0, 0u, 0u};
    };
    pml_gather(g, M, nb, incp, sinc, es, cfh, w_from_src<HG>(src_of), F, F9, nnode, n_int, npml);
  }
}

template <class L>
size_t rec_smem(int Mmax) {
  return (size_t)L::NS * kTile * 4 + 2 * (8 * kTile * 2) + 6 * (size_t)Mmax * 4;
}

template <bool BODY, bool PLASTIC, int HG, bool UNI>
int launch_interior_v(Context &c, cudaStream_t s, const ElemConst32 &k) {
  const ElemGroup<float> &g = c.gi32;
  const size_t sm = rec_smem<RecInterior<BODY, PLASTIC, HG>>(g.max_tile_nodes);
  auto kern = elem_interior_rec<BODY, PLASTIC, HG, UNI>;
  if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
  kern<<<g.ntiles, kTile, sm, s>>>(g, c.vel32, c.dl32, c.F32, c.nnode, k, c.d_err, c.rec0[0]);
  return EQD_OK;
}
template <bool BODY, bool PLASTIC, int HG>
int launch_interior(Context &c, cudaStream_t s, const ElemConst32 &k) {
  return c.gi32.nrec == 1 ? launch_interior_v<BODY, PLASTIC, HG, true>(c, s, k)
                          : launch_interior_v<BODY, PLASTIC, HG, false>(c, s, k);
}

template <bool BODY, bool S0, int HG, bool UNI>
int launch_pml_v(Context &c, cudaStream_t s, const ElemConst32 &k) {
  const ElemGroup<float> &g = c.gp32;
  const size_t sm = rec_smem<RecPml<BODY, S0, HG>>(g.max_tile_nodes);
  auto kern = elem_pml_rec<BODY, S0, HG, UNI>;
  if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
  kern<<<g.ntiles, kTile, sm, s>>>(g, c.vel32, c.dl32, c.F32, c.F9_32, c.nnode, c.n_int, c.npml, k, c.d_err,
                                   c.rec0[1]);
  return EQD_OK;
}
template <bool BODY, bool S0, int HG>
int launch_pml(Context &c, cudaStream_t s, const ElemConst32 &k) {
  return c.gp32.nrec == 1 ? launch_pml_v<BODY, S0, HG, true>(c, s, k) : launch_pml_v<BODY, S0, HG, false>(c, s, k);
}

template <int HG>
int launch_hg(Context &c, cudaStream_t s, const ElemConst32 &k, bool interior) {
  const bool body = (c.sc.rdampm != 0.0) || (c.sc.C_elastic == 0);
  const bool plastic = (c.sc.C_elastic == 0);
  if (interior) {
    if (plastic) return body ? launch_interior<true, true, HG>(c, s, k) : launch_interior<false, true, HG>(c, s, k);
    return body ? launch_interior<true, false, HG>(c, s, k) : launch_interior<false, false, HG>(c, s, k);
  }
  const bool s0 = c.gp32.stress0 != nullptr;
  if (body) return s0 ? launch_pml<true, true, HG>(c, s, k) : launch_pml<true, false, HG>(c, s, k);
  return s0 ? launch_pml<false, true, HG>(c, s, k) : launch_pml<false, false, HG>(c, s, k);
}

}  // namespace

int record_length(int hg, bool body) {
  const int n = (hg == 2 ? TabCommon<2>::STR : TabCommon<1>::STR) + (body ? 8 : 0);
  static_assert(TabCommon<1>::STR + 8 <= kRecMax, "record longer than RecordParam");
  return (n + 3) / 4 * 4;
}

int launch_elements_rec(Context &c, cudaStream_t s, const ElemConst32 &k, bool interior) {
  return c.sc.C_hg == 2 ? launch_hg<2>(c, s, k, interior) : launch_hg<1>(c, s, k, interior);
}

}  // namespace eqd
