// Element kernels of the binary32 form, streamed layout: every element has its own geometry and
// material tables (used when the mesh has too many distinct element records for the
// record-indexed layout of kernels_elem32r.cu).
//
// Tables are component-major with a row stride `ld` padded to whole tiles, so one
// (component, tile) chunk is 512 contiguous, 512-byte aligned bytes.  Per tile (CTA):
//   tables : one elected thread arms an mbarrier with the tile's byte count and issues one bulk
//            copy (cp.async.bulk, TMA engine) per table component plus one for the tile's
//            incidence list, into shared memory;
//   stage  : meanwhile all threads gather the binary32 copies of velocity and (u + rdampk v) of
//            the tile's nodes into shared memory;
//   element: one thread per element computes its forces from shared memory into per-(corner,
//            element) slots (elem32_common.cuh);
//   gather : one thread per tile node sums its incidences with Kahan-compensated binary32 and adds
//            the result to the node force with one L2 reduction per component.
#include "elem32_common.cuh"

namespace eqd {

using namespace e32;

namespace {

template <bool BODY, bool PLASTIC, int HG>
struct SlabInterior : TabCommon<HG> {
  using B = TabCommon<HG>;
  static constexpr int EM = B::STR + 6;                  // 8 lumped corner masses
  static constexpr int POR = EM + (BODY ? 8 : 0);        // 1 pore pressure
  static constexpr int N = POR + (PLASTIC ? 1 : 0);      // rows copied
  // per-(corner, element) forces [3][8]: over the hourglass vectors when there are some
  static constexpr int FS = HG == 1 ? B::PHI : N;
  static constexpr int NS = HG == 1 ? N : N + 24;        // rows in shared memory
  static constexpr bool IDS = false;  // node ids staged in shared memory
};
template <bool BODY, bool S0, int HG>
struct SlabPml : TabCommon<HG> {
  using B = TabCommon<HG>;
  static constexpr int AB = B::STR + 15;                 // 6 PML factors a_k, b_k
  static constexpr int ST0 = AB + 6;                     // 6 initial stress
  static constexpr int EM = ST0 + (S0 ? 6 : 0);          // 8 lumped corner masses
  static constexpr int N = EM + (BODY ? 8 : 0);
  static constexpr int FS = HG == 1 ? B::PHI : N;
  static constexpr int ES = B::STR;                      // 6 split-stress sums over the stress rows
  static constexpr int NS = HG == 1 ? N : N + 24;
  static constexpr bool IDS = true;  // node ids staged in shared memory
};

// Table source reading column `col` of the staged slab.
template <class L>
struct SlabSrc {
  const float *tab;
  int col;
  __device__ float g(int row) const { return tab[row * kTile + col]; }
  __device__ float em(int a) const { return tab[(L::EM + a) * kTile + col]; }
  __device__ float str(int i) const { return tab[(L::STR + i) * kTile + col]; }
  __device__ float por() const { return tab[L::POR * kTile + col]; }
  __device__ float st0(int i) const { return tab[(L::ST0 + i) * kTile + col]; }
  __device__ float pa(int k) const { return tab[(L::AB + k) * kTile + col]; }
  __device__ float pb(int k) const { return tab[(L::AB + 3 + k) * kTile + col]; }
};

template <int HG>
__device__ __forceinline__ void copy_common(float *tab, const ElemGroup<float> &g, int ld, int e0,
                                            unsigned long long *bar) {
  using C = TabCommon<HG>;
  copy_rows(tab, C::SHP, g.shp, 24, ld, e0, bar);
  if (HG == 1) {
    copy_rows(tab, C::PHI, g.phi, 32, ld, e0, bar);
    copy_rows(tab, C::SS, g.ss, 6, ld, e0, bar);
  } else {
    copy_rows(tab, C::HGC, g.hgcoef, 1, ld, e0, bar);
  }
  copy_rows(tab, C::DET, g.detw, 1, ld, e0, bar);
  copy_rows(tab, C::LAM, g.lam, 1, ld, e0, bar);
  copy_rows(tab, C::MU, g.mu, 1, ld, e0, bar);
}

template <bool BODY, bool PLASTIC, int HG>
__global__ void __launch_bounds__(kTile)
    elem_interior_f32(ElemGroup<float> g, const float *__restrict__ vel32, const float *__restrict__ dl32,
                      float *__restrict__ F, int nnode, ElemConst32 k, int *__restrict__ err) {
  using L = SlabInterior<BODY, PLASTIC, HG>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar;
  const int Mmax = g.max_tile_nodes;
  float *tab = reinterpret_cast<float *>(smem);
  const TileSmem ts = tile_smem(tab + L::NS * kTile, Mmax, false);
  unsigned short *sinc = ts.sinc, *slot_of = ts.slot_of;
  float *sv = ts.sv, *sd = ts.sd;
  const int tid = threadIdx.x;
  const int live = g.tile_ne[blockIdx.x];  // elements of this tile (its first slots)
  const int e0 = blockIdx.x * kTile;
  const int ld = g.ld;
  if (tid == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, (unsigned)(L::N * kTile * 4 + 8 * kTile * 2));
    bulk_g2s(sinc, g.tile_inc + (size_t)blockIdx.x * kTile * 8, 8 * kTile * 2, &bar);
    copy_common<HG>(tab, g, ld, e0, &bar);
    copy_rows(tab, L::STR, g.stress, 6, ld, e0, &bar);
    if (BODY) copy_rows(tab, L::EM, g.em, 8, ld, e0, &bar);
    if (PLASTIC) copy_rows(tab, L::POR, g.porep, 1, ld, e0, &bar);
  }
  __syncthreads();  // barrier initialised before anyone polls it
  int nb;
  const int M = stage_nodes(g, blockIdx.x, vel32, dl32, nnode, Mmax, ts, nb);
  const bool ok = mbar_wait_bounded(&bar, err);
  const unsigned short *incp = ts.sincp;
  if (__syncthreads_or(!ok)) return;  // the whole CTA skips the tile if any thread gave up
  build_slots(incp, M, sinc, slot_of);  // reads the staged pointers of other threads
  __syncthreads();
  const int e = e0 + tid;
  float *fs = tab + L::FS * kTile;
  int sl[8];
  load_slots(slot_of, tid, sl);
  if (tid < live)
    interior_element<BODY, PLASTIC, HG, false>(SlabSrc<L>{tab, tid}, sv, sd, Mmax, sl, tid, k,
                                        PLASTIC ? g.pstrain + e : nullptr, g.stress + e, (size_t)ld, fs);
  __syncthreads();
  interior_gather(g, M, nb, incp, sinc, fs, F, nnode, ts.sids);
}

template <bool BODY, bool S0, int HG>
__global__ void __launch_bounds__(kTile)
    elem_pml_f32(ElemGroup<float> g, const float *__restrict__ vel32, const float *__restrict__ dl32,
                 float *__restrict__ F, float *__restrict__ F9, int nnode, int n_int, int npml,
                 ElemConst32 k, int *__restrict__ err) {
  using L = SlabPml<BODY, S0, HG>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar;
  const int Mmax = g.max_tile_nodes;
  float *tab = reinterpret_cast<float *>(smem);
  const TileSmem ts = tile_smem(tab + L::NS * kTile, Mmax, true);
  unsigned short *sinc = ts.sinc, *slot_of = ts.slot_of;
  float *sv = ts.sv, *sd = ts.sd;
  const int tid = threadIdx.x;
  const int live = g.tile_ne[blockIdx.x];  // elements of this tile (its first slots)
  const int e0 = blockIdx.x * kTile;
  const int ld = g.ld;
  if (tid == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, (unsigned)(L::N * kTile * 4 + 8 * kTile * 2));
    bulk_g2s(sinc, g.tile_inc + (size_t)blockIdx.x * kTile * 8, 8 * kTile * 2, &bar);
    copy_common<HG>(tab, g, ld, e0, &bar);
    copy_rows(tab, L::STR, g.stress, 15, ld, e0, &bar);
    copy_rows(tab, L::AB, g.pml_ab, 6, ld, e0, &bar);
    if (S0) copy_rows(tab, L::ST0, g.stress0, 6, ld, e0, &bar);
    if (BODY) copy_rows(tab, L::EM, g.em, 8, ld, e0, &bar);
  }
  __syncthreads();
  int nb;
  const int M = stage_nodes(g, blockIdx.x, vel32, dl32, nnode, Mmax, ts, nb);
  const bool ok = mbar_wait_bounded(&bar, err);
  const unsigned short *incp = ts.sincp;
  if (__syncthreads_or(!ok)) return;  // the whole CTA skips the tile if any thread gave up
  build_slots(incp, M, sinc, slot_of);  // reads the staged pointers of other threads
  __syncthreads();
  const int e = e0 + tid;
  float *cfh = tab + L::FS * kTile;
  float *es = tab + L::ES * kTile;
  int sl[8];
  load_slots(slot_of, tid, sl);
  if (tid < live)
    pml_element<BODY, S0, HG>(SlabSrc<L>{tab, tid}, sv, sd, Mmax, sl, tid, k, g.stress + e, (size_t)ld,
                              es, cfh);
  __syncthreads();
  auto src_of = [&](int el) { return SlabSrc<L>{tab, el}; };
  pml_gather(g, M, nb, incp, sinc, es, cfh, w_from_src<HG>(src_of), F, F9, nnode, n_int, npml, ts.sids);
}

template <class L>
size_t slab_smem(int Mmax) {
  return (size_t)L::NS * kTile * 4 + tile_smem_bytes(Mmax, L::IDS);
}

template <bool BODY, bool PLASTIC, int HG>
int launch_interior32(Context &c, cudaStream_t s, const ElemConst32 &k) {
  const ElemGroup<float> &g = c.gi32;
  const size_t sm = slab_smem<SlabInterior<BODY, PLASTIC, HG>>(g.max_tile_nodes);
  auto kern = elem_interior_f32<BODY, PLASTIC, HG>;
  if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
  kern<<<g.ntiles, kTile, sm, s>>>(g, c.vel32, c.dl32, c.F32, c.nnode, k, c.d_err);
  return EQD_OK;
}

template <bool BODY, bool S0, int HG>
int launch_pml32(Context &c, cudaStream_t s, const ElemConst32 &k) {
  const ElemGroup<float> &g = c.gp32;
  const size_t sm = slab_smem<SlabPml<BODY, S0, HG>>(g.max_tile_nodes);
  auto kern = elem_pml_f32<BODY, S0, HG>;
  if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
  kern<<<g.ntiles, kTile, sm, s>>>(g, c.vel32, c.dl32, c.F32, c.F9_32, c.nnode, c.n_int, c.npml, k, c.d_err);
  return EQD_OK;
}

template <int HG>
int launch_streamed(Context &c, cudaStream_t s, const ElemConst32 &k, bool interior) {
  const bool body = (c.sc.rdampm != 0.0) || (c.sc.C_elastic == 0);
  const bool plastic = (c.sc.C_elastic == 0);
  if (interior) {
    if (plastic) return body ? launch_interior32<true, true, HG>(c, s, k) : launch_interior32<false, true, HG>(c, s, k);
    return body ? launch_interior32<true, false, HG>(c, s, k) : launch_interior32<false, false, HG>(c, s, k);
  }
  const bool s0 = c.gp32.stress0 != nullptr;
  if (body) return s0 ? launch_pml32<true, true, HG>(c, s, k) : launch_pml32<true, false, HG>(c, s, k);
  return s0 ? launch_pml32<false, true, HG>(c, s, k) : launch_pml32<false, false, HG>(c, s, k);
}

}  // namespace

int tile_size_interior() { return kTile; }
int tile_size_pml() { return kTile; }

int launch_elements_f32(Context &c, cudaStream_t s, const ElemConst &kd, int part) {
  const e32::ElemConst32 k{(float)kd.dt, (float)kd.rdampk, (float)kd.rdampm, (float)kd.gz,
                           (float)kd.ccosphi, (float)kd.sinphi, (float)kd.relax};
  const int hg = c.sc.C_hg == 2 ? 2 : 1;
  for (int grp = 0; grp < 2; ++grp) {
    if ((grp == 0 && part == 1) || (grp == 1 && part == 0)) continue;
    const ElemGroup<float> &g = grp == 0 ? c.gi32 : c.gp32;
    if (g.ne == 0) continue;
    int rc;
    if (g.nrec > 0) rc = launch_elements_rec(c, s, k, grp == 0);
    else rc = hg == 2 ? launch_streamed<2>(c, s, k, grp == 0) : launch_streamed<1>(c, s, k, grp == 0);
    if (rc) return rc;
  }
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

}  // namespace eqd
