// Record-layout element bodies of the binary32 form, shared by the per-group kernels
// (kernels_elem32r.cu) and the persistent ensemble kernel (kernels_fault.cu): the shared-memory
// row layouts of a tile, the table sources and the interior / PML tile bodies.  A body uses the
// CTA's dynamic shared memory for one tile; a caller that runs several tiles in one CTA
// separates them with __syncthreads().
#pragma once
#include <type_traits>

#include "elem32_common.cuh"

namespace eqd {
namespace {

using namespace e32;

// Shared-memory rows of a tile (kTile floats each).  Every per-element row is read and written
// only by the thread of its element (column), and each thread reads its copied rows before it
// writes its per-corner forces, so the force rows overlay the copied rows: a CTA needs
// max(copied, 24) rows instead of copied + 24 (more CTAs per SM).
template <bool BODY, bool PLASTIC, int HG, bool QM = false>
struct RecInterior {
  static constexpr int REM = TabCommon<HG>::STR;         // record: 8 corner masses after mu
  static constexpr int QC = REM + (BODY ? 8 : 0);        // record: 5 Q constants (QM)
  static constexpr int STR = 0;                          // shared-memory rows: 6 stress
                                                         // (+ 6 Q memory variables)
  static constexpr int POR = QM ? 12 : 6;                // 1 pore pressure
  static constexpr int RID = POR + (PLASTIC ? 1 : 0);    // record index (u32)
  static constexpr int N = RID + 1;                      // rows copied
  static constexpr int FS = 0;                           // 24 rows of per-corner forces (overlay)
  static constexpr int NS = 24;
  static constexpr bool IDS = false;                     // node ids re-read by the gather
  // the slot table (2 KB, copied with the tile) overlays force rows 20-23: word column e of the
  // table holds element e's slots only (slot_index), and each thread reads its slots before it
  // writes its own forces there; 10 CTAs per SM instead of 9 on C1
  static constexpr int SLOT = 20;
  static_assert(N <= SLOT, "slot rows clear of the copied rows");
};
// UNI (a group with one record): no record-index row, so the tile needs 512 bytes less shared
// memory (the 8th CTA per SM on C1).
template <bool BODY, bool S0, int HG, bool UNI = false>
struct RecPml {
  static constexpr int REM = TabCommon<HG>::STR;
  static constexpr int RID = 0;                          // record index (u32): read again by the
                                                         // node gather, so never overlaid (not UNI)
  static constexpr int STR = UNI ? 0 : 1;                // 15 split-field stress
  static constexpr int ST0 = STR + 15;                   // 6 initial stress
  static constexpr int N = ST0 + (S0 ? 6 : 0);
  static constexpr int ES = STR;                         // 6 split-stress sums over the stress rows
  static constexpr int FS = ES + 6;                      // 24 rows of per-corner forces (overlay)
  static constexpr int NS = FS + 24;
  // the slot table (built on the device) overlays force rows 20-23, clear of the copied rows: word
  // column e holds element e's slots only, and each thread reads its slots before it writes its
  // own forces there.  With the PML axis indices read from global memory by each element's thread
  // (not copied), a tile needs 3 KB less shared memory than with both in rows of their own.
  static constexpr int SLOT = FS + 20;
  static constexpr bool IDS = false;                     // node ids re-read by the gather: staging
                                                         // them costs a CTA per SM
  static_assert(NS >= N, "copied rows fit");
  static_assert(SLOT >= N, "slot rows clear of the copied rows");
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
  __device__ float q(int i) const { return __ldg(rec + L::QC + i); }
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
  __device__ float q(int i) const { return r.v[L::QC + i]; }
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

// Everything one record-layout element launch reads: the group, the node arrays, the constants
// and (UNI) the group's single record.
struct ElemArgs32 {
  ElemGroup<float> g;
  const float *vel32, *dl32;
  float *F, *F9;
  int nnode, n_int, npml;
  int *err;
  ElemConst32 k;
  RecordParam rp;
};

template <bool BODY, bool PLASTIC, int HG, bool UNI, bool QM>
__device__ __forceinline__ void interior_rec_body(const ElemArgs32 &a, int tile) {
  using L = RecInterior<BODY, PLASTIC, HG, QM>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar;
  const ElemGroup<float> &g = a.g;
  const int Mmax = g.max_tile_nodes;
  float *tab = reinterpret_cast<float *>(smem);
  const TileSmem ts = tile_smem(tab + L::NS * kTile, Mmax, L::IDS,
                                reinterpret_cast<unsigned short *>(tab + L::SLOT * kTile));
  unsigned short *sinc = ts.sinc, *slot_of = ts.slot_of;
  float *sv = ts.sv, *sd = ts.sd;
  const int tid = threadIdx.x;
  const int live = g.tile_ne[tile];  // elements of this tile (its first slots)
  const int e0 = tile * kTile;
  const int ld = g.ld;
  if (tid == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, (unsigned)(L::N * kTile * 4 + 2 * (8 * kTile * 2)));
    bulk_g2s(sinc, g.tile_inc + (size_t)tile * kTile * 8, 8 * kTile * 2, &bar);
    bulk_g2s(slot_of, g.tile_slot + (size_t)tile * kTile * 8, 8 * kTile * 2, &bar);
    copy_rows(tab, L::STR, g.stress, QM ? 12 : 6, ld, e0, &bar);
    if (PLASTIC) copy_rows(tab, L::POR, g.porep, 1, ld, e0, &bar);
    copy_rows(tab, L::RID, g.rec_id, 1, ld, e0, &bar);
  }
  __syncthreads();
  int nb;
  const int M = stage_nodes(g, tile, a.vel32, a.dl32, a.nnode, Mmax, ts, nb);
  const bool ok = mbar_wait_bounded(&bar, a.err);
  const unsigned short *incp = ts.sincp;
  if (__syncthreads_or(!ok)) return;  // the whole CTA skips the tile if any thread gave up
  const int e = e0 + tid;
  float *fs = tab + L::FS * kTile;
  int sl[8];
  load_slots(slot_of, tid, sl);  // column tid of the slot rows is this thread's own: no barrier
  if (tid < live) {
    double *ps = PLASTIC ? g.pstrain + e : nullptr;
    if (UNI) {
      const UniSrc<L> S{a.rp, tab, tid, nullptr, 0, 0u, 0u};
      interior_element<BODY, PLASTIC, HG, QM>(S, sv, sd, Mmax, sl, tid, a.k, ps, g.stress + e, (size_t)ld, fs);
    } else {
      const RecSrc<L> S{g.rec + (size_t)row_u32(tab, L::RID, tid) * g.rec_len, tab, tid, nullptr, 0, 0u, 0u};
      interior_element<BODY, PLASTIC, HG, QM>(S, sv, sd, Mmax, sl, tid, a.k, ps, g.stress + e, (size_t)ld, fs);
    }
  }
  __syncthreads();
  interior_gather(g, M, nb, incp, sinc, fs, a.F, a.nnode, ts.sids);
}

template <bool BODY, bool S0, int HG, bool UNI>
__device__ __forceinline__ void pml_rec_body(const ElemArgs32 &a, int tile) {
  using L = RecPml<BODY, S0, HG, UNI>;
  using C = TabCommon<HG>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar;
  // UNI: per corner a the negated det * shape gradient of the group's record as the pairs of
  // pml_gather: (wx, wx), (wy, wy), (wz, wz), (wx, wy)
  __shared__ __align__(16) float cw2[8][8];
  const ElemGroup<float> &g = a.g;
  const int Mmax = g.max_tile_nodes;
  float *tab = reinterpret_cast<float *>(smem);
  const TileSmem ts = tile_smem(tab + L::NS * kTile, Mmax, L::IDS,
                                reinterpret_cast<unsigned short *>(tab + L::SLOT * kTile));
  unsigned short *sinc = ts.sinc, *slot_of = ts.slot_of;
  float *sv = ts.sv, *sd = ts.sd;
  const int tid = threadIdx.x;
  const int live = g.tile_ne[tile];  // elements of this tile (its first slots)
  const int e0 = tile * kTile;
  const int ld = g.ld;
  if (tid == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, (unsigned)(L::N * kTile * 4 + 8 * kTile * 2));
    bulk_g2s(sinc, g.tile_inc + (size_t)tile * kTile * 8, 8 * kTile * 2, &bar);
    copy_rows(tab, L::STR, g.stress, 15, ld, e0, &bar);
    if (S0) copy_rows(tab, L::ST0, g.stress0, 6, ld, e0, &bar);
    if (!UNI) copy_rows(tab, L::RID, g.rec_id, 1, ld, e0, &bar);
  }
  if (UNI && tid < 64) {
    const int ca = tid >> 3, k = tid & 7;
    const int comp = k < 6 ? (k >> 1) : (k - 6);  // x x y y z z x y
    cw2[ca][k] = -(a.rp.v[C::DET] * a.rp.v[C::SHP + 3 * ca + comp]);
  }
  __syncthreads();
  int nb;
  const int M = stage_nodes(g, tile, a.vel32, a.dl32, a.nnode, Mmax, ts, nb);
  const bool ok = mbar_wait_bounded(&bar, a.err);
  const unsigned short *incp = ts.sincp;
  if (__syncthreads_or(!ok)) return;  // the whole CTA skips the tile if any thread gave up
  build_slots(incp, M, sinc, slot_of);  // reads the staged pointers of other threads (the slot table
  __syncthreads();                      // costs the PML pass more as a copy than built here)
  const int e = e0 + tid;
  float *cfh = tab + L::FS * kTile;
  float *es = tab + L::ES * kTile;
  const float *rec = g.rec;
  const int rlen = g.rec_len;
  int sl[8];
  load_slots(slot_of, tid, sl);
  if (tid < live) {
    const unsigned ab01 = __ldg(g.ab_id + e), ab2 = __ldg(g.ab_id + (size_t)ld + e);
    if (UNI) {
      const UniSrc<L> S{a.rp, tab, tid, g.ab_tab, g.ab_stride, ab01, ab2};
      pml_element<BODY, S0, HG>(S, sv, sd, Mmax, sl, tid, a.k, g.stress + e, (size_t)ld, es, cfh);
    } else {
      const RecSrc<L> S{rec + (size_t)row_u32(tab, L::RID, tid) * rlen, tab, tid, g.ab_tab, g.ab_stride,
                        ab01, ab2};
      pml_element<BODY, S0, HG>(S, sv, sd, Mmax, sl, tid, a.k, g.stress + e, (size_t)ld, es, cfh);
    }
  }
  __syncthreads();
  if (UNI) {
    auto w2_of = [&](int, int c, float2 &wxx, float2 &wyy, float2 &wzz, float2 &wxy) {
      const float4 p = *reinterpret_cast<const float4 *>(&cw2[c][0]);
      const float4 q = *reinterpret_cast<const float4 *>(&cw2[c][4]);
      wxx = make_float2(p.x, p.y);
      wyy = make_float2(p.z, p.w);
      wzz = make_float2(q.x, q.y);
      wxy = make_float2(q.z, q.w);
    };
    pml_gather(g, M, nb, incp, sinc, es, cfh, w2_of, a.F, a.F9, a.nnode, a.n_int, a.npml, ts.sids);
  } else {
    auto src_of = [&](int el) {
      return RecSrc<L>{rec + (size_t)row_u32(tab, L::RID, el) * rlen, tab, el, nullptr, 0, 0u, 0u};
    };
    pml_gather(g, M, nb, incp, sinc, es, cfh, w_from_src<HG>(src_of), a.F, a.F9, a.nnode, a.n_int, a.npml,
               ts.sids);
  }
}

__device__ __forceinline__ int elem_batch_member(const int *__restrict__ start, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
template <class L, class = void>
struct SlotOver : std::false_type {};
template <class L>
struct SlotOver<L, std::void_t<decltype(L::SLOT)>> : std::true_type {};

template <class L>
size_t rec_smem(int Mmax) {
  return (size_t)L::NS * kTile * 4 + tile_smem_bytes(Mmax, L::IDS, SlotOver<L>::value);
}

}  // namespace
}  // namespace eqd
