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

#include "elem32_common.cuh"

namespace eqd {

using namespace e32;

namespace {

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
template <bool BODY, bool S0, int HG>
struct RecPml {
  static constexpr int REM = TabCommon<HG>::STR;
  static constexpr int RID = 0;                          // record index (u32): read again by the
                                                         // node gather, so never overlaid
  static constexpr int ABID = 1;                         // 2 rows of PML axis indices (u32)
  static constexpr int STR = 3;                          // 15 split-field stress
  static constexpr int ST0 = 18;                         // 6 initial stress
  static constexpr int N = ST0 + (S0 ? 6 : 0);
  static constexpr int ES = STR;                         // 6 split-stress sums over the stress rows
  static constexpr int FS = ES + 6;                      // 24 rows of per-corner forces (overlay)
  static constexpr int NS = FS + 24;
  static constexpr bool IDS = false;                     // node ids re-read by the gather: staging
                                                         // them costs the 8th CTA per SM
  static_assert(NS >= N, "copied rows fit");
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
  using L = RecPml<BODY, S0, HG>;
  using C = TabCommon<HG>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar;
  // UNI: per corner a the negated det * shape gradient of the group's record as the pairs of
  // pml_gather: (wx, wx), (wy, wy), (wz, wz), (wx, wy)
  __shared__ __align__(16) float cw2[8][8];
  const ElemGroup<float> &g = a.g;
  const int Mmax = g.max_tile_nodes;
  float *tab = reinterpret_cast<float *>(smem);
  const TileSmem ts = tile_smem(tab + L::NS * kTile, Mmax, L::IDS);
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
    copy_rows(tab, L::RID, g.rec_id, 1, ld, e0, &bar);
    copy_rows(tab, L::ABID, g.ab_id, 2, ld, e0, &bar);
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
    const unsigned ab01 = row_u32(tab, L::ABID, tid), ab2 = row_u32(tab, L::ABID + 1, tid);
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
__device__ __forceinline__ int elem_batch_member(const int *__restrict__ start, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
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

template <class L, class = void>
struct SlotOver : std::false_type {};
template <class L>
struct SlotOver<L, std::void_t<decltype(L::SLOT)>> : std::true_type {};

template <class L>
size_t rec_smem(int Mmax) {
  return (size_t)L::NS * kTile * 4 + tile_smem_bytes(Mmax, L::IDS, SlotOver<L>::value);
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
  const size_t sm = rec_smem<RecPml<BODY, S0, HG>>(a.g.max_tile_nodes);
  if (a.g.nrec == 1) {
    auto kern = elem_pml_rec<BODY, S0, HG, true>;
    if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
    kern<<<a.g.ntiles, kTile, sm, s>>>(a);
  } else {
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
