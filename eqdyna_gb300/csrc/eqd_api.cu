// C ABI of the GB300 hot path (include/eqdyna_gb300.h): converts the Fortran globalvar arrays
// into the device layout, drives the per-step kernels (optionally through a CUDA graph) and
// copies results back into the Fortran arrays.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "eqd_device.cuh"
#include "elem32_common.cuh"
#include "mlp_common.cuh"
#include "setup_device.h"

#include <omp.h>
#include <parallel/algorithm>

#include <algorithm>
#include <memory>
#include <chrono>
#include <tuple>
#include <unordered_map>

namespace eqd {
ElemConst make_elem_const(const Context &c);
int tile_size_interior();
int tile_size_pml();
int record_length(int hg, bool body, bool q);
}  // namespace eqd

using namespace eqd;

struct eqd_context {
  Context c;
  double init_ms[8] = {};  // wall time of the setup phases (eqd_gpu_init_times)
  // host-side maps between the Fortran numbering and the device layout
  std::vector<int> node_dev, node_orig;          // original node (0-based) <-> device id (-1: padding)
  int nnode_mesh = 0;                            // nodes of the mesh (device nodes include padding)
  std::vector<int> gi_orig, gp_orig;             // device element slot -> original element
  std::vector<int> pair_station_col;             // on-fault station columns
  std::vector<double> times;                     // timeElapsed after n steps
  std::vector<unsigned char> split_node;         // device node -> 1 for a split (fault) node
  int nftmx = 0;
};

namespace {

constexpr int kNodeBlock = 32;  // device node ranges are padded to multiples of this

template <typename T>
int dalloc(Context &c, T *&p, size_t n) {
  p = nullptr;
  if (n == 0) return EQD_OK;
  void *q = nullptr;
  if (cudaMalloc(&q, n * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    return EQD_ERR_OOM;
  }
  c.allocs.push_back(q);
  p = static_cast<T *>(q);
  return EQD_OK;
}

// Allocator whose vectors leave new elements uninitialised: the element setup writes every entry
// of its scratch tables (tens of GB on C1-size meshes) once, in parallel, so a zero-fill in the
// constructor would only double the host memory traffic (single-threaded).
template <class T>
struct NoInitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <class U>
  NoInitAlloc(const NoInitAlloc<U> &) noexcept {}
  template <class U>
  void construct(U *) noexcept {}
  template <class U, class... Args>
  void construct(U *p, Args &&...args) {
    ::new ((void *)p) U(std::forward<Args>(args)...);
  }
};
template <class T>
using Scratch = std::vector<T, NoInitAlloc<T>>;
// n zeros written by all host threads (a value-initialised vector is filled by one)
Scratch<double> zeros64(size_t n) {
  Scratch<double> v(n);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)n; ++i) v[i] = 0.0;
  return v;
}

template <typename T, class A>
int dupload(Context &c, T *&p, const std::vector<T, A> &h) {
  int rc = dalloc(c, p, h.size());
  if (rc) return rc;
  if (!h.empty() && cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    return EQD_ERR_CUDA;
  return EQD_OK;
}

#define RC(x)                 \
  do {                        \
    int rc_ = (x);            \
    if (rc_) return rc_;      \
  } while (0)

// PML damping profile at a point (comdampv, src/comdampv.f90:1-120, for nodes: non-strict
// corner tests; calcPMLElemKU, src/assembleGlobalKU.f90:139-213, for element centres: strict).
// Region 14 compares y against xmax in both reference routines; that comparison is kept.
void pml_damping(const eqd_scalars &s, double x, double y, double z, bool element, double d[3]) {
  const double xmax0 = s.PMLb[0], xmin0 = s.PMLb[1], ymax0 = s.PMLb[2], ymin0 = s.PMLb[3], zmin0 = s.PMLb[4];
  auto GE = [&](double p, double q) { return element ? p > q : p >= q; };
  auto LE = [&](double p, double q) { return element ? p < q : p <= q; };
  d[0] = d[1] = d[2] = 0.0;
  const bool below = element ? (z < zmin0) : (z <= zmin0);
  const bool above = z > zmin0;
  if (!below && !above) return;
  d[2] = below ? std::fabs(z - zmin0) : 0.0;
  if (GE(x, xmax0) && GE(y, ymax0)) { d[0] = std::fabs(x - xmax0); d[1] = std::fabs(y - ymax0); }
  else if (GE(x, xmax0) && LE(y, ymin0)) { d[0] = std::fabs(x - xmax0); d[1] = std::fabs(y - ymin0); }
  else if (LE(x, xmin0) && LE(y, ymin0)) { d[0] = std::fabs(x - xmin0); d[1] = std::fabs(y - ymin0); }
  else if (LE(x, xmin0) && GE(y, xmax0)) { d[0] = std::fabs(x - xmin0); d[1] = std::fabs(y - ymax0); }
  else if (GE(x, xmax0) && y > ymin0 && y < ymax0) { d[0] = std::fabs(x - xmax0); }
  else if (LE(y, ymin0) && x > xmin0 && x < xmax0) { d[1] = std::fabs(y - ymin0); }
  else if (LE(x, xmin0) && y > ymin0 && y < ymax0) { d[0] = std::fabs(x - xmin0); }
  else if (GE(y, ymax0) && x > xmin0 && x < xmax0) { d[1] = std::fabs(y - ymax0); }
  const double cell[3] = {s.PMLb[5], s.PMLb[6], s.PMLb[7]};
  for (int k = 0; k < 3; ++k) {
    const double delta = s.nPML * cell[k];
    d[k] = 3.0 * s.vmaxPML / 2.0 / delta * std::log(1.0 / s.R) * std::pow(d[k] / delta, 2.0);
  }
}

// Coarse-grained memory-variable constants for one mechanism (qconstant, src/qconstant.f90:3-35,
// after Liu & Archuleta 2006): relaxation time, weight and the unrelaxed-modulus factor.
void q_constants(double Q, int k, double &tau, double &wk, double &c1) {
  static const float taus[8] = {1.72333e-3f, 1.80701e-3f, 5.38887e-3f, 1.99322e-2f,
                                8.49833e-2f, 4.09335e-1f, 2.05951f, 13.2629f};
  static const float alf[8] = {1.66958e-2f, 3.81644e-2f, 9.84666e-3f, -1.36803e-2f,
                               -2.85125e-2f, -5.37309e-2f, -6.65035e-2f, -1.33696e-1f};
  static const float bet[8] = {8.98758e-2f, 6.84635e-2f, 9.67052e-2f, 1.20172e-1f,
                               1.30728e-1f, 1.38746e-1f, 1.40705e-1f, 2.14647e-1f};
  double kap = 3.071f + 1.433f * std::pow(Q, (double)-1.158f) * std::log(Q / 5);
  kap = kap / (1 + 0.415f * Q);
  wk = kap * (kap * (double)alf[k - 1] + (double)bet[k - 1]);
  tau = taus[k - 1];
  const double w2 = 2.0 * 4.0 * std::atan(1.0);
  const double den = 1.0 + (tau * w2) * (tau * w2);
  const double ak0 = 1.0 - wk * 8.0 / den, bk0 = wk * 8.0 * w2 * tau / den;
  const double r = std::pow(ak0 * ak0 + bk0 * bk0, -0.5);
  c1 = 0.5 * r * (1.0 + ak0 * r);
}

// Integer cell coordinates of the elements of a group (x, y, z per element).
struct ElemBins {
  std::vector<int> f;  // [3 * m]
  bool ok = true;      // every coordinate non-negative and small enough for the sort key
};

// Bins of width h (the group's median element extent per axis) from the lowest centroid.
ElemBins bins_by_spacing(const std::vector<double> &c, const double lo[3], const double h[3]) {
  const size_t m = c.size() / 3;
  ElemBins b;
  b.f.resize(3 * m);
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (size_t i = 0; i < m; ++i)
    for (int k = 0; k < 3; ++k) {
      const long v = (long)std::floor((c[3 * i + k] - lo[k]) / h[k] + 0.5);
      if (v < 0 || v > (1l << 24)) bad = 1;
      b.f[3 * i + k] = (int)v;
    }
  b.ok = !bad;
  return b;
}

// Bins by rank: x and z are the ranks of the element's centroid among the group's distinct
// centroid positions along that axis (positions equal to h / 1000), y the rank among the distinct
// y positions of its (x, z) layer.  A structured layer of stretched cells (PML) gets one bin per
// cell and no gaps, where bins of one width merge small cells and skip over large ones.
ElemBins bins_by_rank(const std::vector<double> &c, const double lo[3], const double h[3]) {
  const size_t m = c.size() / 3;
  ElemBins b;
  b.f.resize(3 * m);
  std::vector<long long> q(3 * m);
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < m; ++i)
    for (int k = 0; k < 3; ++k) q[3 * i + k] = std::llround((c[3 * i + k] - lo[k]) / (h[k] * 1e-3));
  for (int k = 0; k < 3; k += 2) {
    std::vector<long long> u(m);
    for (size_t i = 0; i < m; ++i) u[i] = q[3 * i + k];
    __gnu_parallel::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < m; ++i)
      b.f[3 * i + k] = (int)(std::lower_bound(u.begin(), u.end(), q[3 * i + k]) - u.begin());
  }
  std::vector<std::tuple<int, int, long long, size_t>> order(m);
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < m; ++i) order[i] = std::make_tuple(b.f[3 * i], b.f[3 * i + 2], q[3 * i + 1], i);
  __gnu_parallel::sort(order.begin(), order.end());
  int r = 0;
  for (size_t j = 0; j < m; ++j) {
    if (j > 0) {
      const bool same_layer = std::get<0>(order[j]) == std::get<0>(order[j - 1]) &&
                              std::get<1>(order[j]) == std::get<1>(order[j - 1]);
      r = !same_layer ? 0 : (std::get<2>(order[j]) != std::get<2>(order[j - 1]) ? r + 1 : r);
    }
    b.f[3 * std::get<3>(order[j]) + 1] = r;
  }
  return b;
}

// Fraction of the slots that hold an element when every brick of bx x by x bz bins starts a new
// tile (bricks of at most one tile): elements / (tile x sum over bricks of ceil(count / tile)).
double live_fraction(const ElemBins &b, int bx, int by, int bz, int tile) {
  const size_t m = b.f.size() / 3;
  int n0 = 0, n1 = 0, n2 = 0;
#pragma omp parallel for schedule(static) reduction(max : n0, n1, n2)
  for (size_t i = 0; i < m; ++i) {
    n0 = std::max(n0, b.f[3 * i] + 1);
    n1 = std::max(n1, b.f[3 * i + 1] + 1);
    n2 = std::max(n2, b.f[3 * i + 2] + 1);
  }
  const long nb0 = (n0 + bx - 1) / bx, nb1 = (n1 + by - 1) / by, nb2 = (n2 + bz - 1) / bz;
  if (nb0 * nb1 * nb2 > (1l << 31)) return 0.0;
  std::vector<int> cnt((size_t)(nb0 * nb1 * nb2), 0);
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < m; ++i) {
    const size_t k = ((size_t)(b.f[3 * i] / bx) * nb2 + b.f[3 * i + 2] / bz) * nb1 + b.f[3 * i + 1] / by;
#pragma omp atomic
    ++cnt[k];
  }
  long tiles = 0;
#pragma omp parallel for schedule(static) reduction(+ : tiles)
  for (size_t k = 0; k < cnt.size(); ++k) tiles += (cnt[k] + tile - 1) / tile;
  return tiles > 0 ? (double)m / ((double)tiles * tile) : 0.0;
}

// Spatially compact order of an element group for the binary32 tiles: elements are binned in
// bricks of bx x bz x by cells and ordered brick by brick, x-major, then z, then y inside a brick.
// Works for any mesh; structured meshes give exact bricks.  When a brick is at most one tile, a
// brick that does not fill its last tile (at a mesh edge) is followed by empty slots (-1) up to the
// tile boundary, so that every tile holds one brick: without them one partial brick shifts every
// later tile across two bricks (C1 at dx = 200 m: 262 instead of 214 distinct nodes per tile on
// average, 311 at most).
//
// Cells are bins of the group's median element extent.  When that leaves a tenth or more of the
// slots empty (C3: wedge cells hold two elements, so a brick that the dipping fault crosses spills
// into a second tile; its PML shell has stretched cells that the bins merge or skip), the order
// also tries bins by rank (bins_by_rank) and bricks a little smaller than the tuned one, and keeps
// the candidate with the most live slots.  Returns the live fraction chosen (0 when the order
// could not be built).
// Every node id of the connectivity in 1 .. nnode: checked before anything reads coordinates or
// builds tables through it (a bad id would index past the caller's arrays).
bool connectivity_in_range(const eqd_host_arrays &a) {
  const long long n8 = 8 * (long long)a.nelem;
  const int nn = a.nnode;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (long long q = 0; q < n8; ++q) bad |= (a.nodeElemIdRelation[q] < 1 || a.nodeElemIdRelation[q] > nn);
  return !bad;
}

double brick_order(const eqd_host_arrays &a, std::vector<int> &ids, int bx, int bz, int by, int tile) {
  const size_t m = ids.size();
  if (m == 0) return 1.0;
  std::vector<double> c(3 * m), ext(3 * m);
  double lo0 = 1e300, lo1 = 1e300, lo2 = 1e300;
#pragma omp parallel for schedule(static) reduction(min : lo0, lo1, lo2)
  for (size_t i = 0; i < m; ++i) {
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300}, sum[3] = {0, 0, 0};
    for (int q = 0; q < 8; ++q) {
      const double *x = a.meshCoor + 3 * (size_t)(a.nodeElemIdRelation[8 * (size_t)ids[i] + q] - 1);
      for (int k = 0; k < 3; ++k) {
        mn[k] = std::min(mn[k], x[k]);
        mx[k] = std::max(mx[k], x[k]);
        sum[k] += x[k];
      }
    }
    for (int k = 0; k < 3; ++k) {
      c[3 * i + k] = sum[k] / 8.0;
      ext[3 * i + k] = mx[k] - mn[k];
    }
    lo0 = std::min(lo0, c[3 * i]);
    lo1 = std::min(lo1, c[3 * i + 1]);
    lo2 = std::min(lo2, c[3 * i + 2]);
  }
  const double lo[3] = {lo0, lo1, lo2};
  double h[3];
  for (int k = 0; k < 3; ++k) {
    std::vector<double> e(m);
    for (size_t i = 0; i < m; ++i) e[i] = ext[3 * i + k];
    std::nth_element(e.begin(), e.begin() + m / 2, e.end());
    h[k] = e[m / 2] > 0 ? e[m / 2] : 1.0;
  }
  if (bx > 32 || bz > 32 || by > 64) return 0.0;  // not representable: caller keeps the input order
  ElemBins bins = bins_by_spacing(c, lo, h);
  if (!bins.ok) return 0.0;
  const bool pad = bx * by * bz <= tile;
  double live = pad ? live_fraction(bins, bx, by, bz, tile) : 1.0;
  if (pad && live < 0.9) {
    ElemBins rank = bins_by_rank(c, lo, h);
    int best_b = 0, sx = bx, sy = by, sz = bz;
    // candidates: the tuned brick and bricks a little smaller along each axis (down to three
    // quarters), so that wedge pairs fit in a tile.  (Trying every brick shape of one tile as well
    // picked, on C3's interior, a shape with 4 % more live slots but 15 % more node gathers per
    // element, and a slower pass: 2.28 -> 2.40 ms.)
    for (int which = 0; which < 2; ++which) {
      const ElemBins &b = which == 0 ? bins : rank;
      for (int cx = bx; cx >= std::max(1, (3 * bx + 3) / 4); --cx)
        for (int cz = bz; cz >= std::max(1, (3 * bz + 3) / 4); --cz)
          for (int cy = by; cy >= std::max(1, (3 * by + 3) / 4); --cy) {
            const double f = live_fraction(b, cx, cy, cz, tile);
            if (f > live + 1e-9) {
              live = f;
              best_b = which;
              sx = cx, sy = cy, sz = cz;
            }
          }
    }
    if (best_b == 1) bins = std::move(rank);
    bx = sx, by = sy, bz = sz;
  }
  // sort key (brick x, brick z, brick y, then x, z, y inside the brick, then the element), packed
  // into 64 bits: 16 bits per brick index, 16 for the position inside the brick
  std::vector<std::pair<uint64_t, int>> keys(m);
  int wide = 0;
#pragma omp parallel for schedule(static) reduction(| : wide)
  for (size_t i = 0; i < m; ++i) {
    const long fx = bins.f[3 * i], fy = bins.f[3 * i + 1], fz = bins.f[3 * i + 2];
    const uint64_t b0 = (uint64_t)(fx / bx), b1 = (uint64_t)(fz / bz), b2 = (uint64_t)(fy / by);
    const uint64_t w = (uint64_t)(fx % bx) << 11 | (uint64_t)(fz % bz) << 6 | (uint64_t)(fy % by);
    if (b0 > 0xffff || b1 > 0xffff || b2 > 0xffff) wide = 1;
    keys[i] = {b0 << 48 | b1 << 32 | b2 << 16 | w, ids[i]};
  }
  if (wide) return 0.0;
  __gnu_parallel::sort(keys.begin(), keys.end());
  if (!pad) {
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < m; ++i) ids[i] = keys[i].second;
    return 1.0;
  }
  ids.clear();
  ids.reserve(m + m / 8);
  for (size_t i = 0; i < m; ++i) {
    const bool new_brick = i > 0 && (keys[i].first >> 16) != (keys[i - 1].first >> 16);
    if (new_brick)
      while (ids.size() % tile) ids.push_back(-1);
    ids.push_back(keys[i].second);
  }
  return live;
}

// Tile metadata: per tile its distinct nodes and, per node, the incidences (corner * tile + local
// element) in ascending order.  Nodes are ordered by incidence count (most first), then by device
// id, so the 32 nodes of a warp in the gather loop have (nearly) the same trip count.
int build_tiles(Context &c, ElemGroup<float> &g, const Scratch<int> &conn_dev, int tile) {
  const int m = g.ne;
  g.tile = tile;
  g.ntiles = (m + tile - 1) / tile;
  const int nt = g.ntiles;
  std::vector<unsigned short> inc((size_t)nt * tile * 8, 0), slot((size_t)nt * tile * 8, 0);
  std::vector<std::vector<int>> tnodes(nt);
  std::vector<std::vector<unsigned short>> tincp(nt);
  std::vector<int> tile_ne(nt, 0);
  int maxM = 0, bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : maxM) reduction(| : bad)
  for (int t = 0; t < nt; ++t) {
    const int e0 = t * tile, e1 = std::min(m, e0 + tile);
    std::vector<std::pair<int, int>> pairs;
    pairs.reserve((size_t)(e1 - e0) * 8);
    for (int e = e0; e < e1; ++e) {
      if (conn_dev[e] < 0) continue;  // empty slot
      if (e - e0 != tile_ne[t]) bad = 1;  // the elements of a tile must be its first slots
      ++tile_ne[t];
      for (int q = 0; q < 8; ++q) pairs.push_back({conn_dev[(size_t)q * m + e], q * tile + (e - e0)});
    }
    std::sort(pairs.begin(), pairs.end());
    std::vector<std::pair<size_t, size_t>> runs;  // [first, last) of each node's incidences
    for (size_t k = 0; k < pairs.size(); ++k)
      if (k == 0 || pairs[k].first != pairs[k - 1].first) runs.push_back({k, k});
    for (size_t r = 0; r < runs.size(); ++r) runs[r].second = r + 1 < runs.size() ? runs[r + 1].first : pairs.size();
    std::stable_sort(runs.begin(), runs.end(), [](const std::pair<size_t, size_t> &x, const std::pair<size_t, size_t> &y) {
      return x.second - x.first > y.second - y.first;
    });
    const size_t base = (size_t)t * tile * 8;
    std::vector<int> &nodes = tnodes[t];
    std::vector<unsigned short> &incp = tincp[t];
    nodes.reserve(runs.size());
    incp.reserve(runs.size() + 1);
    size_t k = 0;
    for (const auto &run : runs) {
      const unsigned short j = (unsigned short)nodes.size();
      nodes.push_back(pairs[run.first].first);
      incp.push_back((unsigned short)k);
      for (size_t q = run.first; q < run.second; ++q) {
        inc[base + k++] = (unsigned short)pairs[q].second;
        slot[base + e32::slot_index(pairs[q].second)] = j;
      }
    }
    incp.push_back((unsigned short)pairs.size());
    maxM = std::max(maxM, (int)runs.size());
  }
  std::vector<int> node_ptr(nt + 1, 0), incp_off(nt + 1, 0);
  for (int t = 0; t < nt; ++t) {
    node_ptr[t + 1] = node_ptr[t] + (int)tnodes[t].size();
    incp_off[t + 1] = incp_off[t] + (int)tincp[t].size();
  }
  std::vector<int> nodes(node_ptr[nt]);
  std::vector<unsigned short> incp(incp_off[nt]);
#pragma omp parallel for schedule(static)
  for (int t = 0; t < nt; ++t) {
    std::copy(tnodes[t].begin(), tnodes[t].end(), nodes.begin() + node_ptr[t]);
    std::copy(tincp[t].begin(), tincp[t].end(), incp.begin() + incp_off[t]);
  }
  if (bad) return EQD_ERR_INPUT;
  g.max_tile_nodes = std::max(maxM, 1);
  g.ne_live = 0;
  for (int t = 0; t < nt; ++t) g.ne_live += tile_ne[t];
  g.sum_tile_nodes = node_ptr[nt];
  int rc;
  if ((rc = dupload(c, g.tile_ne, tile_ne))) return rc;
  if ((rc = dupload(c, g.tile_node_ptr, node_ptr))) return rc;
  if ((rc = dupload(c, g.tile_nodes, nodes))) return rc;
  if ((rc = dupload(c, g.tile_incp, incp))) return rc;
  if ((rc = dupload(c, g.tile_incp_off, incp_off))) return rc;
  if ((rc = dupload(c, g.tile_inc, inc))) return rc;
  if ((rc = dupload(c, g.tile_slot, slot))) return rc;
  return EQD_OK;
}

template <class A>
Scratch<float> to_f32(const std::vector<double, A> &v) {
  Scratch<float> out(v.size());
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)v.size(); ++i) out[i] = (float)v[i];
  return out;
}

// Distinct binary32 element records: open addressing over a 64-bit hash of the record's bits.
class RecordDict {
 public:
  explicit RecordDict(int len) : len_(len), slots_(1024, -1) {}
  int len() const { return len_; }
  long size() const { return (long)hash_.size(); }
  const std::vector<float> &rows() const { return rows_; }
  // index of record r (len() floats), added when new; -1 when r is new and `cap` records exist
  long find_or_add(const float *r, long cap) {
    const uint64_t h = hash(r);
    size_t mask = slots_.size() - 1;
    for (size_t i = h & mask;; i = (i + 1) & mask) {
      const long q = slots_[i];
      if (q < 0) {
        if (size() >= cap) return -1;
        slots_[i] = size();
        hash_.push_back(h);
        rows_.insert(rows_.end(), r, r + len_);
        if (2 * hash_.size() > slots_.size()) grow();
        return size() - 1;
      }
      if (hash_[q] == h && std::memcmp(&rows_[(size_t)q * len_], r, (size_t)len_ * 4) == 0) return q;
    }
  }

 private:
  uint64_t hash(const float *r) const {
    uint64_t h = 0x9E3779B97F4A7C15ull;
    for (int k = 0; k < len_; ++k) {
      uint32_t w;
      std::memcpy(&w, r + k, 4);
      h = (h ^ w) * 0x100000001B3ull;
      h ^= h >> 29;
    }
    return h;
  }
  void grow() {
    std::vector<long> ns(slots_.size() * 2, -1);
    const size_t mask = ns.size() - 1;
    for (long q = 0; q < size(); ++q) {
      size_t i = hash_[q] & mask;
      while (ns[i] >= 0) i = (i + 1) & mask;
      ns[i] = q;
    }
    slots_.swap(ns);
  }
  int len_;
  std::vector<long> slots_;
  std::vector<uint64_t> hash_;
  std::vector<float> rows_;
};

// Auto layout: record-indexed when a group's distinct records fit in a third of the 129 MB L2
// (48 MB: C3's sheared and stretched cells have ~100k records of ~280 bytes per element group at
// dx = 100 m) and there are at most half as many records as elements.
constexpr long kAutoRecordBytes = 48l << 20;
inline long auto_max_records(int record_floats) { return kAutoRecordBytes / (4l * record_floats); }

// binary32 copy of a component-major table [ncomp][m] with its rows padded with zeros to stride ld
template <class V>
Scratch<float> to_f32_rows(const V &v, size_t m, size_t ld) {
  const size_t nc = v.size() / m;
  Scratch<float> out(nc * ld);
#pragma omp parallel for schedule(static)
  for (long long qi = 0; qi < (long long)(nc * ld); ++qi) {
    const size_t q = (size_t)qi / ld, i = (size_t)qi % ld;
    out[qi] = i < m ? (float)v[q * m + i] : 0.f;  // rows padded to ld with zeros
  }
  return out;
}

int validate(const eqd_scalars *s, const eqd_host_arrays *a) {
  if (!s || !a) return EQD_ERR_INPUT;
  if (a->nnode <= 0 || a->nelem <= 0 || a->neq <= 0) return EQD_ERR_INPUT;
  if (!a->nodeElemIdRelation || !a->elemTypeArr || !a->eqNumIndexArr || !a->eqNumStartIndexLoc ||
      !a->numOfDofPerNodeArr || !a->meshCoor || !a->mat || !a->stressArr || !a->stressCompIndexArr ||
      !a->v1 || !a->velArr || !a->dispArr || !a->nodalForceArr)
    return EQD_ERR_INPUT;
  // the per-element tables and nodal masses: all given, or none (then built on the device)
  const int given = !!a->eleshp + !!a->eledet + !!a->ss + !!a->phi + !!a->nodalMassArr + !!a->fnms;
  if (given != 0 && given != 6) return EQD_ERR_INPUT;
  if (given == 0 && a->elemass) return EQD_ERR_INPUT;
  if (s->dt <= 0.0 || s->nstep < 0) return EQD_ERR_INPUT;
  if (s->C_hg != 1 && s->C_hg != 2) return EQD_ERR_UNSUPPORTED;
  if (a->ntotft != 1 && a->ntotft != 0) return EQD_ERR_UNSUPPORTED;
  if (s->friclaw < 1 || s->friclaw > 5) return EQD_ERR_INPUT;
  // the reference stops on Q with plasticity (src/warning.f90:6-9, stop 1001)
  if (s->C_Q == 1 && s->C_elastic == 0) return EQD_ERR_UNSUPPORTED;
  if (s->C_Q < 0 || s->C_Q > 2) return EQD_ERR_INPUT;
  return EQD_OK;
}

// Tables of a group's elements (ids, -1 for an empty slot) computed on the device from the mesh
// and copied into the group's host rows (shp[q * m + i] ...), in chunks of device scratch.
template <class V>
int group_tables_from_device(const DeviceMesh &dm, const std::vector<int> &ids, int m, double w, V &shp, V &phi,
                             V &ss, V &detw, V *em) {
  if (m <= 0) return EQD_OK;
  const int cn = std::min(m, 1 << 22);
  double *d = nullptr;
  int *did = nullptr;
  const size_t rows = 24 + 32 + 6 + 1 + 8;
  if (cudaMalloc(&d, rows * cn * sizeof(double)) != cudaSuccess || cudaMalloc(&did, cn * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    if (d) cudaFree(d);
    return EQD_ERR_OOM;
  }
  int rc = EQD_OK;
  double *dshp = d, *dphi = d + 24 * (size_t)cn, *dss = dphi + 32 * (size_t)cn, *ddet = dss + 6 * (size_t)cn;
  double *dem = ddet + cn;
  for (int i0 = 0; i0 < m && !rc; i0 += cn) {
    const int n = std::min(cn, m - i0);
    if (cudaMemcpy(did, ids.data() + i0, n * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
      rc = EQD_ERR_CUDA;
      break;
    }
    if ((rc = device_group_tables(dm, did, n, cn, w, dshp, ddet, em ? dem : nullptr, dss, dphi, 0))) break;
    auto get = [&](double *dst, const double *src, int nrows) {
      for (int q = 0; q < nrows && !rc; ++q)
        if (cudaMemcpy(dst + (size_t)q * m + i0, src + (size_t)q * cn, n * sizeof(double), cudaMemcpyDeviceToHost) !=
            cudaSuccess)
          rc = EQD_ERR_CUDA;
    };
    get(shp.data(), dshp, 24);
    get(phi.data(), dphi, 32);
    get(ss.data(), dss, 6);
    get(detw.data(), ddet, 1);
    if (em) get(em->data(), dem, 8);
  }
  cudaFree(d);
  cudaFree(did);
  return rc;
}

// Device node order: the 3-DOF nodes, then the 12-DOF (PML) nodes, each range padded to whole
// blocks of kNodeBlock with inert nodes (1/m = 0, in no element, no force, state 0).  Every
// component of a node array (stride nnode) and of a PML array (stride npml) then starts on a
// 128-byte boundary and every warp of the node update reads and writes whole sectors: on C1 the
// update runs 5 % faster than with the mesh's counts.  Within the ranges the node update tells its
// node classes by index: split (fault) nodes of the first fault first among the 3-DOF nodes, PML
// nodes with equations before the fixed ones (src/driver.f90:141-144).  Within a class the mesh
// order is kept.
struct NodeOrder {
  std::vector<int> orig;  // device node -> 0-based mesh node, -1 for padding
  int n_split = 0, n_int = 0, npml_live = 0;
};
int device_node_order(const eqd_host_arrays &a, NodeOrder &o) {
  const int nn = a.nnode;
  if (nn <= 0 || !a.numOfDofPerNodeArr || !a.eqNumStartIndexLoc || !a.eqNumIndexArr) return EQD_ERR_INPUT;
  auto eq1 = [&](int j) -> int {  // 0-based node -> 1-based equation of its first DOF, or <= 0
    const int loc = a.eqNumStartIndexLoc[j] + 1;
    if (loc < 1 || loc > a.size_eqidx) return -2;
    return a.eqNumIndexArr[loc - 1];
  };
  const int npair0 = (a.ntotft >= 1 && a.nftnd) ? a.nftnd[0] : 0;
  if (npair0 > 0 && !a.nsmp) return EQD_ERR_INPUT;
  std::vector<unsigned char> split_mesh(nn, 0);
  for (int i = 0; i < npair0; ++i)
    for (int k = 0; k < 2; ++k) {
      const int node = a.nsmp[2 * (size_t)i + k];
      if (node < 1 || node > nn) return EQD_ERR_INPUT;
      split_mesh[node - 1] = 1;
    }
  // class of each node (0 split 3-DOF, 1 other 3-DOF, 2 PML with equations, 3 fixed PML), then a
  // stable counting scatter into the device order
  Scratch<unsigned char> klass(nn);
  long long count[4] = {0, 0, 0, 0};
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : count[:4]) reduction(| : bad)
  for (int j = 0; j < nn; ++j) {
    const int dof = a.numOfDofPerNodeArr[j];
    unsigned char k = 0;
    if (dof == 3) k = split_mesh[j] ? 0 : 1;
    else if (dof == 12) k = eq1(j) > 0 ? 2 : 3;
    else bad = 1;
    klass[j] = k;
    ++count[k];
  }
  if (bad) return EQD_ERR_INPUT;
  auto up = [](long long x) { return (x + kNodeBlock - 1) / kNodeBlock * kNodeBlock; };
  o.n_split = (int)count[0];
  o.n_int = (int)up(count[0] + count[1]);
  o.npml_live = (int)count[2];
  const long long total = o.n_int + up(count[2] + count[3]);
  long long cursor[4] = {0, count[0], o.n_int, o.n_int + count[2]};
  o.orig.assign((size_t)total, -1);
  for (int j = 0; j < nn; ++j) o.orig[(size_t)cursor[klass[j]]++] = j;
  return EQD_OK;
}

int build_device_state(eqd_context &X, const eqd_scalars &s, const eqd_host_arrays &a) {
  auto t_last = std::chrono::steady_clock::now();
  auto mark = [&](int k) {
    const auto t = std::chrono::steady_clock::now();
    X.init_ms[k] += std::chrono::duration<double, std::milli>(t - t_last).count();
    t_last = t;
  };
  Context &c = X.c;
  c.sc = s;
  const int nn = a.nnode, ne = a.nelem;
  X.nnode_mesh = nn;
  c.nelem = ne;
  c.neq = a.neq;
  c.nstep = s.nstep;
  c.size_stress = a.size_stress;
  auto eq = [&](int node, int k) -> int {  // 1-based node, 1-based DOF -> 1-based eq or -1
    const int loc = a.eqNumStartIndexLoc[node - 1] + k;
    if (loc < 1 || loc > a.size_eqidx) return -2;
    return a.eqNumIndexArr[loc - 1];
  };
  // Without host tables the element tables and nodal masses are built on the device from the mesh
  // (setup_device.cu), bit for bit the host's: a node's mass is the value of each of its equations
  // in nodalMassArr and its fnms.
  if (!connectivity_in_range(a)) return EQD_ERR_INPUT;
  const bool dev_tables = a.eleshp == nullptr;
  std::unique_ptr<DeviceMesh> dmesh;
  std::vector<double> dev_mass;
  if (dev_tables) {
    dmesh.reset(new DeviceMesh());
    RC(dmesh->upload(a));
    RC(device_nodal_mass(a, *dmesh, dev_mass));
  }
  auto eq_mass = [&](int node, int e) { return dev_tables ? dev_mass[node - 1] : a.nodalMassArr[e - 1]; };
  auto node_fnms = [&](int node) { return dev_tables ? dev_mass[node - 1] : a.fnms[node - 1]; };
  // ---- nodes ----
  {
    NodeOrder o;
    RC(device_node_order(a, o));
    X.node_orig.swap(o.orig);
    c.n_split = o.n_split;
    c.n_int = o.n_int;
    c.npml_live = o.npml_live;
  }
  X.node_dev.assign(nn, -1);
#pragma omp parallel for schedule(static)
  for (int d = 0; d < (int)X.node_orig.size(); ++d)
    if (X.node_orig[d] >= 0) X.node_dev[X.node_orig[d]] = d;
  const int nd = (int)X.node_orig.size();  // device nodes
  c.nnode = nd;
  c.npml = nd - c.n_int;
  const int np_ = c.npml;
  Scratch<double> vel(3 * (size_t)nd), disp(3 * (size_t)nd);  // every entry written below
  Scratch<double> F = zeros64(3 * (size_t)nd), inv_mass = zeros64(nd);
  Scratch<double> F9 = zeros64(9 * (size_t)np_), v9 = zeros64(9 * (size_t)np_), vh = zeros64(3 * (size_t)np_);
  Scratch<double> pml_ab = zeros64(6 * (size_t)np_);
  int bad_ = EQD_OK;
#pragma omp parallel for schedule(static)
  for (int d = 0; d < nd; ++d) {
    const int r_ = [&]() -> int {
      const int j = X.node_orig[d], node = j + 1;
      if (j < 0) {  // padding: zero state, 1/m = 0 (zero forces and PML factors above)
        for (int k = 0; k < 3; ++k) disp[k * (size_t)nd + d] = 0.0, vel[k * (size_t)nd + d] = 0.0;
        return EQD_OK;
      }
      for (int k = 0; k < 3; ++k) disp[k * (size_t)nd + d] = a.dispArr[3 * (size_t)j + k];
      if (d < c.n_int) {
        double m = -1;
        for (int k = 1; k <= 3; ++k) {
          const int e = eq(node, k);
          if (e < 1 || e > a.neq) return EQD_ERR_UNSUPPORTED;  // fixed 3-DOF node: not built
          const double mk = eq_mass(node, e);
          if (k == 1) m = mk;
          else if (mk != m) return EQD_ERR_UNSUPPORTED;  // anisotropic lumped mass: not built
          vel[(k - 1) * (size_t)nd + d] = a.v1[e - 1];
          F[(k - 1) * (size_t)nd + d] = a.nodalForceArr[e - 1];
        }
        if (!(m > 0)) return EQD_ERR_INPUT;
        inv_mass[d] = 1.0 / m;
      } else {
        const int p = d - c.n_int;
        for (int k = 0; k < 3; ++k) vel[k * (size_t)nd + d] = a.velArr[3 * (size_t)j + k];
        const int e1 = eq(node, 1);
        if (e1 > 0) {
          const double m = eq_mass(node, e1);
          if (!(m > 0)) return EQD_ERR_INPUT;
          for (int k = 1; k <= 12; ++k) {
            const int e = eq(node, k);
            if (e < 1 || e > a.neq) return EQD_ERR_UNSUPPORTED;
            if (eq_mass(node, e) != m) return EQD_ERR_UNSUPPORTED;
            if (k <= 9) {
              v9[(k - 1) * (size_t)np_ + p] = a.v1[e - 1];
              F9[(k - 1) * (size_t)np_ + p] = a.nodalForceArr[e - 1];
            } else {
              vh[(k - 10) * (size_t)np_ + p] = a.v1[e - 1];
              F[(k - 10) * (size_t)nd + d] = a.nodalForceArr[e - 1];
            }
          }
          inv_mass[d] = 1.0 / m;
          double dm[3];
          pml_damping(s, a.meshCoor[3 * (size_t)j], a.meshCoor[3 * (size_t)j + 1], a.meshCoor[3 * (size_t)j + 2], false, dm);
          for (int k = 0; k < 3; ++k) {
            pml_ab[k * (size_t)np_ + p] = 1.0 / s.dt - dm[k] / 2.0;
            pml_ab[(3 + k) * (size_t)np_ + p] = 1.0 / (1.0 / s.dt + dm[k] / 2.0);
          }
        } else {
          for (int k = 1; k <= 12; ++k)
            if (eq(node, k) != -1) return EQD_ERR_UNSUPPORTED;  // partially fixed PML node
        }
      }
      return EQD_OK;
    }();
    if (r_) {
#pragma omp critical(eqd_setup_status)
      bad_ = r_;
    }
  }
  if (bad_) return bad_;
  RC(dupload(c, c.vel, vel));
  RC(dupload(c, c.disp, disp));
  RC(dupload(c, c.inv_mass, inv_mass));
  RC(dupload(c, c.vh, vh));
  if (c.fp32) {
    // binary32 form: force sums, PML split velocities, damping and 1/m in binary32
    RC(dupload(c, c.F32, to_f32(F)));
    RC(dupload(c, c.F9_32, to_f32(F9)));
    RC(dupload(c, c.v9_32, to_f32(v9)));
    RC(dupload(c, c.pml_ab32, to_f32(pml_ab)));
    // split (fault) nodes keep binary64 forces and updates: mark them with a negative 1/m and
    // give each a slot (2 i slave, 2 i + 1 master of pair i) in the binary64 force array
    Scratch<float> im32 = to_f32(inv_mass);
    const int npair0 = (a.ntotft >= 1 && a.nftnd) ? a.nftnd[0] : 0;
    std::vector<int> slot(nd, -1);
    std::vector<double> fsplit(3 * (size_t)std::max(2 * npair0, 1), 0.0);
    for (int i = 0; i < npair0; ++i)
      for (int k = 0; k < 2; ++k) {
        const int node = a.nsmp[2 * (size_t)i + k];
        if (node < 1 || node > nn) return EQD_ERR_INPUT;
        const int d = X.node_dev[node - 1];
        if (d >= c.n_int) return EQD_ERR_UNSUPPORTED;
        slot[d] = 2 * i + k;
        im32[d] = -im32[d];
        if (X.split_node.empty()) X.split_node.assign(nd, 0);
        X.split_node[d] = 1;
        for (int q = 0; q < 3; ++q) fsplit[(size_t)q * 2 * npair0 + 2 * i + k] = F[(size_t)q * nd + d];
      }
    RC(dupload(c, c.inv_mass32, im32));
    RC(dupload(c, c.split_slot, slot));
    RC(dupload(c, c.Fsplit, fsplit));
  } else {
    RC(dupload(c, c.F, F));
    RC(dupload(c, c.F9, F9));
    RC(dupload(c, c.v9, v9));
    RC(dupload(c, c.pml_ab, pml_ab));
  }
  c.f_is_acc = 1;

  mark(0);
  // ---- elements ----
  X.gi_orig.clear();
  X.gp_orig.clear();
  for (int e = 0; e < ne; ++e) {
    const int t = a.elemTypeArr[e];
    if (t == 1 || t > 10) X.gi_orig.push_back(e);
    else if (t == 2) X.gp_orig.push_back(e);
    else return EQD_ERR_INPUT;
  }
  const bool body = (s.rdampm != 0.0) || (s.C_elastic == 0);
  if (c.fp32) {
    // Q memory variables in the binary32 form: record-indexed tables only (the Q constants are
    // part of an element's record)
    if (s.C_Q != 0 && c.opt.table_layout == EQD_TABLES_STREAMED) return EQD_ERR_UNSUPPORTED;
    const int ts = c.opt.tile_shape > 0 ? c.opt.tile_shape : (4 | 8 << 8 | 4 << 16);
    const int bx = ts & 255, by = (ts >> 8) & 255, bz = (ts >> 16) & 255;
    // (a mesh wider than 65536 bricks along an axis keeps the input order)
    brick_order(a, X.gi_orig, bx, bz, by, tile_size_interior());
    brick_order(a, X.gp_orig, bx, bz, by, tile_size_pml());
  }
  mark(1);
  for (int grp = 0; grp < 2; ++grp) {
    const std::vector<int> &ids = grp == 0 ? X.gi_orig : X.gp_orig;
    ElemGroup<double> &g = grp == 0 ? c.gi64 : c.gp64;
    const int m = (int)ids.size();
    if (!c.fp32) g.ne = m;
    else (grp == 0 ? c.gi32 : c.gp32).ne = m;
    if (m == 0) continue;
    Scratch<int> conn(8 * (size_t)m);
    Scratch<double> shp(24 * (size_t)m), phi(32 * (size_t)m), ss(6 * (size_t)m), detw(m), lam(m), mu(m);
    const int nstress = grp == 0 ? (s.C_Q != 0 ? 12 : 6) : 15;
    Scratch<double> st(nstress * (size_t)m);
    Scratch<double> st0, pab, em, hg, porep, pstr, qc;
    bool any_s0 = false;
    int s0_any = 0;
    if (grp == 1) st0 = zeros64(6 * (size_t)m), pab = zeros64(6 * (size_t)m);
    if (body) em = zeros64(8 * (size_t)m);
    if (s.C_hg == 2) hg = zeros64(m);
    if (grp == 0 && s.C_elastic == 0) porep = zeros64(m), pstr = zeros64(m);
    if (grp == 0 && s.C_Q != 0) qc = zeros64(5 * (size_t)m);
    int bad_ = EQD_OK;
#pragma omp parallel for schedule(static) reduction(|| : s0_any)
    for (int i = 0; i < m; ++i) {
      const int r_ = [&]() -> int {
        const int e = ids[i];
        if (e < 0) {  // empty slot of the binary32 tiles: no nodes, zero tables
          for (int q = 0; q < 8; ++q) conn[q * (size_t)m + i] = -1;
          for (int q = 0; q < 24; ++q) shp[q * (size_t)m + i] = 0.0;
          for (int q = 0; q < 32; ++q) phi[q * (size_t)m + i] = 0.0;
          for (int q = 0; q < 6; ++q) ss[q * (size_t)m + i] = 0.0;
          for (int q = 0; q < nstress; ++q) st[q * (size_t)m + i] = 0.0;
          detw[i] = lam[i] = mu[i] = 0.0;
          return EQD_OK;
        }
        double ctr[3] = {0, 0, 0};
        for (int q = 0; q < 8; ++q) {
          const int node = a.nodeElemIdRelation[8 * (size_t)e + q];
          if (node < 1 || node > nn) return EQD_ERR_INPUT;
          conn[q * (size_t)m + i] = X.node_dev[node - 1];
          for (int k = 0; k < 3; ++k) ctr[k] += a.meshCoor[3 * (size_t)(node - 1) + k];
        }
        for (double &v : ctr) v /= 8.0;
        if (!dev_tables) {  // (else filled from the device below)
          for (int q = 0; q < 24; ++q) shp[q * (size_t)m + i] = a.eleshp[24 * (size_t)e + q];
          for (int q = 0; q < 32; ++q) phi[q * (size_t)m + i] = a.phi[32 * (size_t)e + q];
          for (int q = 0; q < 6; ++q) ss[q * (size_t)m + i] = a.ss[6 * (size_t)e + q];
          detw[i] = a.eledet[e] * s.w;
        }
        lam[i] = a.mat[3 * (size_t)ne + e];
        mu[i] = a.mat[4 * (size_t)ne + e];
        const int64_t base = a.stressCompIndexArr[e];
        if (base < 0 || base + (grp == 0 ? nstress : 21) > a.size_stress) return EQD_ERR_INPUT;
        for (int q = 0; q < nstress; ++q) st[q * (size_t)m + i] = a.stressArr[base + q];
        if (grp == 1) {
          for (int q = 0; q < 6; ++q) {
            st0[q * (size_t)m + i] = a.stressArr[base + 15 + q];
            s0_any |= (st0[q * (size_t)m + i] != 0.0);
          }
          double dm[3];
          pml_damping(s, ctr[0], ctr[1], ctr[2], true, dm);
          for (int k = 0; k < 3; ++k) {
            pab[k * (size_t)m + i] = 1.0 / s.dt - dm[k] / 2.0;
            pab[(3 + k) * (size_t)m + i] = 1.0 / (1.0 / s.dt + dm[k] / 2.0);
          }
        }
        if (body && !dev_tables) {
          if (!a.elemass) return EQD_ERR_INPUT;
          for (int q = 0; q < 8; ++q) {
            const double m0 = a.elemass[24 * (size_t)e + 3 * q];
            if (a.elemass[24 * (size_t)e + 3 * q + 1] != m0 || a.elemass[24 * (size_t)e + 3 * q + 2] != m0)
              return EQD_ERR_UNSUPPORTED;
            em[q * (size_t)m + i] = m0;
          }
        }
        if (s.C_hg == 2 && !dev_tables)
          hg[i] = 0.25 * s.kapa_hg * a.mat[2 * (size_t)ne + e] * a.mat[e] * std::pow(a.eledet[e] * s.w, 2.0 / 3.0);
        if (grp == 0 && s.C_elastic == 0) {
          porep[i] = a.eleporep ? a.eleporep[e] : 0.0;
          pstr[i] = a.pstrain ? a.pstrain[e] : 0.0;
        }
        if (grp == 0 && s.C_Q != 0) {
          // Q zone and mechanism index from the element centre (src/calcElemKU.f90:78-103); C_Q = 2
          // (extension): Qs = 50 Vs (km/s), Qp = 2 Qs
          const double Qs = s.C_Q == 2 ? 50.0 * a.mat[1 * (size_t)ne + e] / 1000.0 : (ctr[2] > -1000.0 ? 10.0 : 50.0);
          const double Qp = 2.0 * Qs;
          const int ip = (int)((ctr[0] - (s.PMLb[1] + s.dx / 2)) / s.dx + 1);
          const int iq = (int)((ctr[1] - (s.PMLb[3] + s.dx / 2)) / s.dx + 1);
          const int ir = (int)((ctr[2] - (s.PMLb[4] + s.dx / 2)) / s.dx + 1);
          const int kk = 1 + ip % 2 + 2 * (iq % 2) + 4 * (ir % 2);
          if (kk < 1 || kk > 8) return EQD_ERR_INPUT;
          double tau, wkp, wks, cv, cs;
          q_constants(Qp, kk, tau, wkp, cv);
          q_constants(Qs, kk, tau, wks, cs);
          qc[0 * (size_t)m + i] = std::exp(-s.dt / tau);
          qc[1 * (size_t)m + i] = mu[i] * cs;
          qc[2 * (size_t)m + i] = (lam[i] + 2 * mu[i]) * cv;
          qc[3 * (size_t)m + i] = wkp * 8.0;
          qc[4 * (size_t)m + i] = wks * 8.0;
        }
        return EQD_OK;
      }();
      if (r_) {
#pragma omp critical(eqd_setup_status)
        bad_ = r_;
      }
    }
    if (bad_) return bad_;
    if (dev_tables) {
      RC(group_tables_from_device(*dmesh, ids, m, s.w, shp, phi, ss, detw, body ? &em : nullptr));
      if (s.C_hg == 2) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < m; ++i)
          if (ids[i] >= 0)
            hg[i] = 0.25 * s.kapa_hg * a.mat[2 * (size_t)ne + ids[i]] * a.mat[ids[i]] * std::pow(detw[i], 2.0 / 3.0);
      }
    }
    any_s0 = s0_any;
    if (c.fp32 && grp == 1 && !X.split_node.empty()) {  // does a PML element touch a split node?
      int touch = 0;
#pragma omp parallel for schedule(static) reduction(| : touch)
      for (long long q = 0; q < 8 * (long long)m; ++q)
        if (conn[q] >= 0 && X.split_node[conn[q]]) touch = 1;
      c.pml_touches_split = touch;
    }
    mark(2);
    if (c.fp32) {
      ElemGroup<float> &h = grp == 0 ? c.gi32 : c.gp32;
      RC(build_tiles(c, h, conn, grp == 0 ? tile_size_interior() : tile_size_pml()));
      mark(3);
      h.ld = h.ntiles * h.tile;  // whole tiles: every (component, tile) chunk is one aligned bulk copy
      const size_t um = (size_t)m, ld = (size_t)h.ld;
      // record-indexed layout: one record per distinct binary32 (geometry, material) combination
      const int layout = c.opt.table_layout;
      bool use_rec = layout != EQD_TABLES_STREAMED;
      const bool qm = grp == 0 && s.C_Q != 0;
      RecordDict dict(record_length(s.C_hg, body, qm));
      std::vector<unsigned> rid, abid;
      std::vector<float> abt;
      if (use_rec) {
        // per-thread dictionaries over contiguous chunks, merged in chunk order
        const long cap = (layout == EQD_TABLES_RECORDS || qm) ? (long)m : std::min<long>(auto_max_records(dict.len()), m / 2 + 1);
        rid.assign(ld, 0u);
        const int T = std::max(1, omp_get_max_threads());
        std::vector<RecordDict> local(T, RecordDict(dict.len()));
        std::vector<int> overflow(T, 0);
#pragma omp parallel for schedule(static, 1) num_threads(T)
        for (int t = 0; t < T; ++t) {
          const long long i0 = (long long)m * t / T, i1 = (long long)m * (t + 1) / T;
          std::vector<float> r(dict.len(), 0.f);
          for (long long i = i0; i < i1; ++i) {
            if (ids[i] < 0) {  // empty slot: any record (never read)
              rid[i] = ~0u;
              continue;
            }
            int q = 0;
            for (int k = 0; k < 24; ++k) r[q++] = (float)shp[k * um + i];
            if (s.C_hg == 2) {
              r[q++] = (float)hg[i];
            } else {
              for (int k = 0; k < 32; ++k) r[q++] = (float)phi[k * um + i];
              for (int k = 0; k < 6; ++k) r[q++] = (float)ss[k * um + i];
            }
            r[q++] = (float)detw[i];
            r[q++] = (float)lam[i];
            r[q++] = (float)mu[i];
            if (body)
              for (int k = 0; k < 8; ++k) r[q++] = (float)em[k * um + i];
            if (qm)
              for (int k = 0; k < 5; ++k) r[q++] = (float)qc[k * um + i];
            const long id = local[t].find_or_add(r.data(), cap);
            if (id < 0) {
              overflow[t] = 1;
              break;
            }
            rid[i] = (unsigned)id;
          }
        }
        std::vector<std::vector<unsigned>> to_global(T);
        for (int t = 0; t < T && use_rec; ++t) {
          if (overflow[t]) use_rec = false;
          for (long j = 0; j < local[t].size() && use_rec; ++j) {
            const long id = dict.find_or_add(local[t].rows().data() + (size_t)j * dict.len(), cap);
            if (id < 0) use_rec = false;
            else to_global[t].push_back((unsigned)id);
          }
        }
        if (use_rec) {
#pragma omp parallel for schedule(static, 1) num_threads(T)
          for (int t = 0; t < T; ++t) {
            const long long i0 = (long long)m * t / T, i1 = (long long)m * (t + 1) / T;
            for (long long i = i0; i < i1; ++i) rid[i] = rid[i] == ~0u ? 0u : to_global[t][rid[i]];
          }
        }
      }
      if (use_rec && grp == 1) {  // PML factors: distinct (a_k, b_k) per axis
        abid.assign(2 * ld, 0u);
        std::vector<float> pairs[3];
        std::vector<unsigned> axis_id[3];
        int overflow_ab = 0;
        // the three axes are independent dictionaries: one thread each
#pragma omp parallel for schedule(static, 1) num_threads(3) reduction(| : overflow_ab)
        for (int k = 0; k < 3; ++k) {
          std::unordered_map<uint64_t, unsigned> seen;
          uint64_t last_key = ~0ull;
          unsigned last = 0;
          axis_id[k].assign(m, 0u);
          for (int i = 0; i < m; ++i) {
            const float fa = (float)pab[k * um + i], fb = (float)pab[(3 + k) * um + i];
            uint32_t ba, bb;
            std::memcpy(&ba, &fa, 4);
            std::memcpy(&bb, &fb, 4);
            const uint64_t key = (uint64_t)ba | ((uint64_t)bb << 32);
            if (key != last_key) {
              auto it = seen.find(key);
              if (it != seen.end()) {
                last = it->second;
              } else {
                if ((int)seen.size() >= kPmlAxisMax) { overflow_ab = 1; break; }
                last = (unsigned)seen.size();
                seen.emplace(key, last);
                pairs[k].push_back(fa);
                pairs[k].push_back(fb);
              }
              last_key = key;
            }
            axis_id[k][i] = last;
          }
        }
        if (overflow_ab) use_rec = false;
        if (use_rec) {
#pragma omp parallel for schedule(static)
          for (int i = 0; i < m; ++i) {
            abid[i] = axis_id[0][i] | axis_id[1][i] << 16;
            abid[ld + i] = axis_id[2][i];
          }
        }
        if (use_rec) {
          h.ab_stride = (int)(std::max({pairs[0].size(), pairs[1].size(), pairs[2].size()}) / 2);
          abt.assign(3 * (size_t)h.ab_stride * 2, 0.f);
          for (int k = 0; k < 3; ++k)
            std::copy(pairs[k].begin(), pairs[k].end(), abt.begin() + 2 * (size_t)k * h.ab_stride);
        }
      }
      if (!use_rec && (layout == EQD_TABLES_RECORDS || qm)) return EQD_ERR_UNSUPPORTED;
      if (use_rec) {
        h.nrec = (int)dict.size();
        h.rec_len = dict.len();
        std::copy(dict.rows().begin(), dict.rows().begin() + dict.len(), c.rec0[grp].v);
        RC(dupload(c, h.rec, dict.rows()));
        RC(dupload(c, h.rec_id, rid));
        if (grp == 1) {
          RC(dupload(c, h.ab_id, abid));
          RC(dupload(c, h.ab_tab, abt));
        }
      } else {
        RC(dupload(c, h.shp, to_f32_rows(shp, um, ld)));
        RC(dupload(c, h.phi, to_f32_rows(phi, um, ld)));
        RC(dupload(c, h.ss, to_f32_rows(ss, um, ld)));
        RC(dupload(c, h.detw, to_f32_rows(detw, um, ld)));
        RC(dupload(c, h.lam, to_f32_rows(lam, um, ld)));
        RC(dupload(c, h.mu, to_f32_rows(mu, um, ld)));
        if (grp == 1) RC(dupload(c, h.pml_ab, to_f32_rows(pab, um, ld)));
        if (body) RC(dupload(c, h.em, to_f32_rows(em, um, ld)));
        if (s.C_hg == 2) RC(dupload(c, h.hgcoef, to_f32_rows(hg, um, ld)));
      }
      RC(dupload(c, h.stress, to_f32_rows(st, um, ld)));
      if (grp == 1 && any_s0) RC(dupload(c, h.stress0, to_f32_rows(st0, um, ld)));
      if (!porep.empty()) RC(dupload(c, h.porep, to_f32_rows(porep, um, ld)));
      if (!pstr.empty()) RC(dupload(c, h.pstrain, pstr));
      mark(4);
      continue;
    }
    RC(dupload(c, g.conn, conn));
    RC(dupload(c, g.shp, shp));
    RC(dupload(c, g.phi, phi));
    RC(dupload(c, g.ss, ss));
    RC(dupload(c, g.detw, detw));
    RC(dupload(c, g.lam, lam));
    RC(dupload(c, g.mu, mu));
    RC(dupload(c, g.stress, st));
    if (grp == 1 && any_s0) RC(dupload(c, g.stress0, st0));
    if (grp == 1) RC(dupload(c, g.pml_ab, pab));
    if (body) RC(dupload(c, g.em, em));
    if (s.C_hg == 2) RC(dupload(c, g.hgcoef, hg));
    if (!porep.empty()) RC(dupload(c, g.porep, porep));
    if (!pstr.empty()) RC(dupload(c, g.pstrain, pstr));
    if (!qc.empty()) RC(dupload(c, g.qcoef, qc));
  }
  if (c.fp32) {
    RC(dalloc(c, c.vel32, 3 * (size_t)nd));
    RC(dalloc(c, c.dl32, 3 * (size_t)nd));
    EQD_CUDA_OK(cudaMemset(c.vel32, 0, 3 * (size_t)nd * sizeof(float)));
    EQD_CUDA_OK(cudaMemset(c.dl32, 0, 3 * (size_t)nd * sizeof(float)));
  }

  mark(4);
  // ---- fault ----
  const int npair = (a.ntotft >= 1 && a.nftnd) ? a.nftnd[0] : 0;
  c.npair = npair;
  X.nftmx = a.nftmx;
  if (npair > 0) {
    if (!a.nsmp || !a.un || !a.us || !a.ud || !a.arn || !a.fric || !a.fnft || a.nftmx < npair)
      return EQD_ERR_INPUT;
    std::vector<int> ps(npair), pm(npair);
    std::vector<double> geo(13 * (size_t)npair), fr(100 * (size_t)npair), fn(npair);
    for (int i = 0; i < npair; ++i) {
      const int sl = a.nsmp[2 * (size_t)i], ms = a.nsmp[2 * (size_t)i + 1];
      if (sl < 1 || sl > nn || ms < 1 || ms > nn) return EQD_ERR_INPUT;
      ps[i] = X.node_dev[sl - 1];
      pm[i] = X.node_dev[ms - 1];
      if (ps[i] >= c.n_int || pm[i] >= c.n_int) return EQD_ERR_UNSUPPORTED;  // split node in PML
      for (int k = 0; k < 3; ++k) {
        geo[(0 + k) * (size_t)npair + i] = a.un[3 * (size_t)i + k];
        geo[(3 + k) * (size_t)npair + i] = a.us[3 * (size_t)i + k];
        geo[(6 + k) * (size_t)npair + i] = a.ud[3 * (size_t)i + k];
      }
      geo[9 * (size_t)npair + i] = a.arn[i];
      geo[10 * (size_t)npair + i] = node_fnms(sl);
      geo[11 * (size_t)npair + i] = node_fnms(ms);
      const double *x = a.meshCoor + 3 * (size_t)(sl - 1);
      geo[12 * (size_t)npair + i] = std::sqrt((x[0] - s.xsource) * (x[0] - s.xsource) +
                                              (x[1] - s.ysource) * (x[1] - s.ysource) +
                                              (x[2] - s.zsource) * (x[2] - s.zsource));
      for (int k = 0; k < 100; ++k) fr[k * (size_t)npair + i] = a.fric[100 * (size_t)i + k];
      fn[i] = a.fnft[i];
    }
    RC(dupload(c, c.pair_s, ps));
    RC(dupload(c, c.pair_m, pm));
    RC(dupload(c, c.pair_geo, geo));
    RC(dupload(c, c.fric, fr));
    RC(dupload(c, c.fnft, fn));
    const bool tp = (s.friclaw == 5) || (X.c.opt.record_tp_hist && s.friclaw >= 3);
    if (tp && s.nstep > 0) {
      std::vector<double> h(2 * (size_t)npair * s.nstep, 0.0);
      if (a.onFaultTPHist)
        for (int t = 0; t < s.nstep; ++t)
          for (int i = 0; i < npair; ++i)
            for (int k = 0; k < 2; ++k)
              h[2 * ((size_t)i + (size_t)npair * t) + k] = a.onFaultTPHist[2 * ((size_t)i + (size_t)a.nftmx * t) + k];
      RC(dupload(c, c.tp_hist, h));
    } else if (s.friclaw == 5) {
      return EQD_ERR_INPUT;
    }
  }
  // ---- stations ----
  std::vector<PairStation> onst;
  if (a.numOnFaultSt > 0 && a.anonfs) {
    for (int j = 0; j < a.numOnFaultSt; ++j)
      if (a.anonfs[3 * (size_t)j + 2] == 1 && a.anonfs[3 * (size_t)j] >= 1 && a.anonfs[3 * (size_t)j] <= npair)
        onst.push_back({a.anonfs[3 * (size_t)j] - 1, j});
  }
  c.nOnSt = (int)onst.size();
  RC(dupload(c, c.onst, onst));
  const int ncol = a.numOnFaultSt > 0 ? a.numOnFaultSt : 1;
  if (s.nstep > 0) {
    std::vector<double> oh(12 * (size_t)s.nstep * ncol, 0.0);
    if (a.onFaultQuantHistSCECForm) std::memcpy(oh.data(), a.onFaultQuantHistSCECForm, oh.size() * sizeof(double));
    RC(dupload(c, c.onhist, oh));
  }
  c.nOffRows = 6 * a.numOffFaultSt;
  if (c.nOffRows > 0) {
    if (!a.idhist) return EQD_ERR_INPUT;
    std::vector<int> rows(3 * (size_t)c.nOffRows);
    for (int r = 0; r < c.nOffRows; ++r) {
      const int node = a.idhist[3 * (size_t)r], comp = a.idhist[3 * (size_t)r + 1], type = a.idhist[3 * (size_t)r + 2];
      if (node < 1 || node > nn || comp < 1 || comp > 3 || (type != 1 && type != 2)) return EQD_ERR_UNSUPPORTED;
      rows[r] = X.node_dev[node - 1];
      rows[c.nOffRows + r] = comp - 1;
      rows[2 * c.nOffRows + r] = type;
    }
    RC(dupload(c, c.off_rows, rows));
    if (s.nstep > 0) {
      std::vector<double> hh((size_t)(c.nOffRows + 1) * s.nstep, 0.0);
      if (a.OffFaultStGramSCEC) std::memcpy(hh.data(), a.OffFaultStGramSCEC, hh.size() * sizeof(double));
      RC(dupload(c, c.offhist, hh));
    }
  }
  mark(5);
  // ---- step bookkeeping ----
  RC(dalloc(c, c.d_nt, 1));
  RC(dalloc(c, c.d_nt_c, 1));
  RC(dalloc(c, c.d_err, 1));
  RC(dalloc(c, c.d_stats, 5));
  EQD_CUDA_OK(cudaMemset(c.d_nt, 0, sizeof(int)));
  EQD_CUDA_OK(cudaMemset(c.d_err, 0, sizeof(int)));
  EQD_CUDA_OK(cudaMemset(c.d_stats, 0, 5 * sizeof(unsigned long long)));
  c.nt = 0;
  c.time = s.time0;
  X.times.assign(1, s.time0);
  return EQD_OK;
}

int ensure_times(eqd_context &X, int last_nt) {
  Context &c = X.c;
  if (last_nt + 1 <= c.times_cap) return EQD_OK;
  while ((int)X.times.size() < last_nt + 1 + 256) X.times.push_back(X.times.back() + c.sc.dt);
  double *d = nullptr;
  if (cudaMalloc(&d, X.times.size() * sizeof(double)) != cudaSuccess) return EQD_ERR_OOM;
  if (cudaMemcpy(d, X.times.data(), X.times.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    return EQD_ERR_CUDA;
  if (c.d_times) {
    cudaFree(c.d_times);
    for (auto &p : c.allocs)
      if (p == c.d_times) p = d;
  } else {
    c.allocs.push_back(d);
  }
  c.d_times = d;
  c.times_cap = (int)X.times.size();
  if (c.graph) {  // the graph captured the old pointer
    cudaGraphExecDestroy(c.graph);
    c.graph = nullptr;
  }
  return EQD_OK;
}

// Events of one profiled step: [start, after node, after interior, after PML, after fault].
constexpr int kEventsPerStep = 5;

// The overlapped schedule (binary32 form, no per-launch profiling).  The fault phase of step n
// (thermal pressurization, fault kernel, fric(47) frame) touches only split nodes and fault rows;
// the bulk node update of step n + 1 touches every other node, and the PML element pass (when no
// PML element has a split node) reads and adds to non-split nodes only.  So they run side by side:
// the fault phase on c.side, forked after the interior element pass of step n and joined before the
// split nodes of step n + 1 are updated.  Per step: bulk node update, PML elements || fault phase of
// the previous step; split nodes (and the step number for the fault phase); off-fault station
// rows; surface frame; interior elements.  The last fault phase of a call runs on the main stream,
// so every call ends with the state of a completed step.
int launch_steps_overlapped(Context &c, int nsteps) {
  if (!c.side) {
    // the fault phase is a short chain of latency-bound launches beside a bandwidth-bound one:
    // give it the highest priority so that its blocks are placed first as SM slots free up
    int lo = 0, hi = 0;
    EQD_CUDA_OK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    EQD_CUDA_OK(cudaStreamCreateWithPriority(&c.side, cudaStreamNonBlocking, hi));
    EQD_CUDA_OK(cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming));
    EQD_CUDA_OK(cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming));
  }
  for (int k = 0; k < nsteps; ++k) {
    // the fault phase of the previous step (binary64 transcendentals) is forked after this step's
    // bulk node update, which needs the binary64 pipe too, so that it runs beside the PML pass
    const bool fork = k > 0 && !c.pml_touches_split;
    if (k > 0 && c.pml_touches_split) {
      EQD_CUDA_OK(cudaEventRecord(c.ev_fork, c.stream));
      EQD_CUDA_OK(cudaStreamWaitEvent(c.side, c.ev_fork, 0));
      RC(launch_fault(c, c.side, true));
      RC(launch_output_capture(c, c.side, 2, true));
      EQD_CUDA_OK(cudaEventRecord(c.ev_join, c.side));
    }
    RC(launch_node_update(c, c.stream, true));
    if (fork) {
      EQD_CUDA_OK(cudaEventRecord(c.ev_fork, c.stream));
      EQD_CUDA_OK(cudaStreamWaitEvent(c.side, c.ev_fork, 0));
      RC(launch_fault(c, c.side, true));
      RC(launch_output_capture(c, c.side, 2, true));
      EQD_CUDA_OK(cudaEventRecord(c.ev_join, c.side));
    }
    // the PML elements touch no split node: they run beside the fault phase
    if (!c.pml_touches_split) RC(launch_elements(c, c.stream, 1));
    if (k > 0) EQD_CUDA_OK(cudaStreamWaitEvent(c.stream, c.ev_join, 0));
    RC(launch_split_update(c, c.stream));
    c.f_is_acc = 0;
    RC(launch_station_capture(c, c.stream));
    RC(launch_output_capture(c, c.stream, 1, true));
    RC(launch_elements(c, c.stream, 0));
    if (c.pml_touches_split) RC(launch_elements(c, c.stream, 1));
  }
  RC(launch_fault(c, c.stream, true));
  RC(launch_output_capture(c, c.stream, 2, true));
  return EQD_OK;
}

int launch_step(Context &c, cudaEvent_t *ev = nullptr) {
  if (ev) EQD_CUDA_OK(cudaEventRecord(ev[0], c.stream));
  RC(launch_node_update(c, c.stream));
  c.f_is_acc = 0;
  if (ev) EQD_CUDA_OK(cudaEventRecord(ev[1], c.stream));
  RC(launch_elements(c, c.stream, 0));
  if (ev) EQD_CUDA_OK(cudaEventRecord(ev[2], c.stream));
  RC(launch_elements(c, c.stream, 1));
  if (ev) EQD_CUDA_OK(cudaEventRecord(ev[3], c.stream));
  RC(launch_fault(c, c.stream));
  RC(launch_output_capture(c, c.stream));
  if (ev) EQD_CUDA_OK(cudaEventRecord(ev[4], c.stream));
  return EQD_OK;
}

int ensure_events(Context &c, int nsteps) {
  const size_t need = (size_t)kEventsPerStep * nsteps;
  while (c.prof_events.size() < need) {
    cudaEvent_t e;
    EQD_CUDA_OK(cudaEventCreate(&e));
    c.prof_events.push_back(e);
  }
  return EQD_OK;
}

// Accumulates the profiled times of the last `nsteps` steps (the stream is synchronised).
int accumulate_profile(Context &c, int nsteps) {
  for (int k = 0; k < nsteps; ++k) {
    cudaEvent_t *ev = &c.prof_events[(size_t)kEventsPerStep * k];
    float ms[4];
    for (int q = 0; q < 4; ++q) EQD_CUDA_OK(cudaEventElapsedTime(&ms[q], ev[q], ev[q + 1]));
    float all;
    EQD_CUDA_OK(cudaEventElapsedTime(&all, ev[0], ev[4]));
    c.prof_ms[0] += all;
    c.prof_launches[0] += 1;
    for (int q = 0; q < 4; ++q) c.prof_ms[q + 1] += ms[q];
    c.prof_launches[1] += 1;
    c.prof_launches[2] += (c.gi64.ne > 0 || c.gi32.ne > 0) ? 1 : 0;
    c.prof_launches[3] += (c.gp64.ne > 0 || c.gp32.ne > 0) ? 1 : 0;
    c.prof_launches[4] += (c.npair + c.nOffRows > 0) ? 1 : 0;
  }
  return EQD_OK;
}

// Register-resident FMA chains: 8 independent chains per thread, 2 flops per FMA.
__global__ void fp64_fma_chain(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

constexpr int kGraphSteps = 16;

bool overlapped(const Context &c) { return c.fp32 && !c.profile && !c.opt.sequential_fault; }

// Kernel launches of one step (for the launch counters).
int launches_per_step(const Context &c) {
  const int elem = (c.gi64.ne > 0 || c.gi32.ne > 0 ? 1 : 0) + (c.gp64.ne > 0 || c.gp32.ne > 0 ? 1 : 0);
  const int tp = (c.sc.friclaw == 5 && c.tp_hist) ? 1 : 0;
  const int out = c.out_frames ? 1 : 0;
  if (!overlapped(c)) return 2 + elem + tp + out;
  return 3 + elem + tp + (c.nOffRows > 0 && c.offhist ? 1 : 0) + 2 * out;
}

int build_graph(Context &c) {
  cudaGraph_t g = nullptr;
  EQD_CUDA_OK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
  int rc = EQD_OK;
  if (overlapped(c)) rc = launch_steps_overlapped(c, kGraphSteps);
  else
    for (int k = 0; k < kGraphSteps && rc == EQD_OK; ++k) rc = launch_step(c);
  cudaError_t e = cudaStreamEndCapture(c.stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return EQD_ERR_CUDA;
  e = cudaGraphInstantiate(&c.graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    c.graph = nullptr;
    return EQD_ERR_CUDA;
  }
  c.graph_steps = kGraphSteps;
  return EQD_OK;
}

}  // namespace

extern "C" {

const char *eqd_gpu_status_string(int status) {
  switch (status) {
    case EQD_OK: return "ok";
    case EQD_ERR_INPUT: return "inconsistent or missing input";
    case EQD_ERR_CUDA: return "CUDA runtime error";
    case EQD_ERR_OOM: return "device out of memory";
    case EQD_ERR_NAN: return "NaN velocity";
    case EQD_ERR_UNSUPPORTED: return "unsupported option combination";
    case EQD_ERR_NO_DEVICE: return "no CUDA device";
    case EQD_ERR_TIMEOUT: return "bounded device wait timed out";
    case EQD_ERR_STATE: return "call out of order";
    default: return "unknown status";
  }
}

int eqd_gpu_init(const eqd_scalars *s, const eqd_host_arrays *a, const eqd_options *opt, eqd_context **out) {
  if (!out) return EQD_ERR_INPUT;
  *out = nullptr;
  int rc = validate(s, a);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return EQD_ERR_NO_DEVICE;
  }
  eqd_context *X = new (std::nothrow) eqd_context();
  if (!X) return EQD_ERR_OOM;
  Context &c = X->c;
  if (opt) c.opt = *opt;
  c.device = c.opt.device;
  if (c.device < 0 || c.device >= ndev) {
    delete X;
    return EQD_ERR_INPUT;
  }
  if (cudaSetDevice(c.device) != cudaSuccess) {
    delete X;
    return EQD_ERR_CUDA;
  }
  c.fp32 = (c.opt.precision == EQD_PREC_FP32);
  {  // launch shapes (eqdyna_gb300.autotune chooses them; 0 = default)
    const int ts = c.opt.tile_shape, bx = ts & 255, by = (ts >> 8) & 255, bz = (ts >> 16) & 255;
    const int bn = c.opt.block_node, bf = c.opt.block_fault;
    const bool ok = (ts == 0 || (bx * by * bz == tile_size_interior() && (ts >> 24) == 0)) &&
                    (bn == 0 || bn == 64 || bn == 128 || bn == 256 || bn == 512) &&
                    (bf == 0 || bf == 32 || bf == 64 || bf == 128);
    if (!ok) {
      delete X;
      return EQD_ERR_INPUT;
    }
  }
  rc = build_device_state(*X, *s, *a);
  if (!rc && c.opt.learned_guess) rc = mlp_init(c);
  if (!rc && cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) rc = EQD_ERR_CUDA;
  if (rc) {
    eqd_gpu_finalize(X);
    return rc;
  }
  *out = X;
  return EQD_OK;
}

namespace {
// Queues nsteps steps from nt_begin on the context's stream.
int enqueue_steps(eqd_context *X, int32_t nt_begin, int32_t nsteps, int64_t &launches_out) {
  Context &c = X->c;
  RC(ensure_times(*X, nt_begin + nsteps));
  if (nt_begin != c.nt + 1) {
    const int prev = nt_begin - 1;
    EQD_CUDA_OK(cudaMemcpyAsync(c.d_nt, &prev, sizeof(int), cudaMemcpyHostToDevice, c.stream));
    c.nt = prev;
  }
  int done = 0;
  int64_t launches = 0;
  const int per_step = launches_per_step(c);
  const bool ov = overlapped(c);
  if (c.profile) {
    RC(ensure_events(c, nsteps));
    for (; done < nsteps; ++done) RC(launch_step(c, &c.prof_events[(size_t)kEventsPerStep * done]));
    launches = (int64_t)per_step * nsteps;
  }
  // the first step after init consumes the stored acceleration and runs outside the graph
  if (c.f_is_acc && done < nsteps) {
    RC(ov ? launch_steps_overlapped(c, 1) : launch_step(c));
    ++done;
    launches += per_step;
  }
  if (c.opt.use_graph && nsteps - done >= kGraphSteps) {
    if (!c.graph) RC(build_graph(c));
    while (nsteps - done >= kGraphSteps) {
      EQD_CUDA_OK(cudaGraphLaunch(c.graph, c.stream));
      done += kGraphSteps;
      launches += (int64_t)per_step * kGraphSteps;
    }
  }
  if (ov && done < nsteps) {
    RC(launch_steps_overlapped(c, nsteps - done));
    launches += (int64_t)per_step * (nsteps - done);
    done = nsteps;
  }
  for (; done < nsteps; ++done) {
    RC(launch_step(c));
    launches += per_step;
  }
  EQD_CUDA_OK(cudaGetLastError());
  launches_out = launches;
  return EQD_OK;
}

int err_status(int err) { return (err & 2) ? EQD_ERR_TIMEOUT : (err ? EQD_ERR_NAN : EQD_OK); }
}  // namespace

int eqd_gpu_step(eqd_context *X, int32_t nt_begin, int32_t nsteps) {
  if (!X) return EQD_ERR_STATE;
  if (nsteps < 0 || nt_begin < 1) return EQD_ERR_INPUT;
  if (nsteps == 0) return EQD_OK;
  Context &c = X->c;
  cudaSetDevice(c.device);
  int64_t launches = 0;
  if (c.time_calls) EQD_CUDA_OK(cudaEventRecord(c.call_ev[0], c.stream));
  RC(enqueue_steps(X, nt_begin, nsteps, launches));
  if (c.time_calls) EQD_CUDA_OK(cudaEventRecord(c.call_ev[1], c.stream));
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  EQD_CUDA_OK(cudaGetLastError());
  int err = 0;
  EQD_CUDA_OK(cudaMemcpy(&err, c.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (c.profile) RC(accumulate_profile(c, nsteps));
  if (c.time_calls) {
    float ms = 0.f;
    EQD_CUDA_OK(cudaEventElapsedTime(&ms, c.call_ev[0], c.call_ev[1]));
    c.prof_ms[0] += ms;
    c.prof_launches[0] += nsteps;
  }
  c.nt += nsteps;
  c.time = X->times[c.nt];
  c.launches_last = launches;
  c.elem_updates += (int64_t)c.nelem * nsteps;
  return err_status(err);
}

int eqd_gpu_step_async(eqd_context *X, int32_t nt_begin, int32_t nsteps) {
  if (!X) return EQD_ERR_STATE;
  if (nsteps < 0 || nt_begin < 1) return EQD_ERR_INPUT;
  if (nsteps == 0) return EQD_OK;
  Context &c = X->c;
  if (c.profile) return EQD_ERR_STATE;  // profiling accumulates event times at every step call
  cudaSetDevice(c.device);
  int64_t launches = 0;
  RC(enqueue_steps(X, nt_begin, nsteps, launches));
  c.nt += nsteps;
  c.time = X->times[c.nt];
  c.launches_last = launches;
  c.elem_updates += (int64_t)c.nelem * nsteps;
  return EQD_OK;
}

int eqd_gpu_fetch_fric_rows_async(eqd_context *X, const int32_t *rows, int32_t nrows, double *dst,
                                  int64_t *ticket) {
  if (!X) return EQD_ERR_STATE;
  if (nrows < 1 || !rows || !dst || !ticket) return EQD_ERR_INPUT;
  Context &c = X->c;
  const int np = c.npair;
  for (int r = 0; r < nrows; ++r)
    if (rows[r] < 1 || rows[r] > 100) return EQD_ERR_INPUT;
  cudaSetDevice(c.device);
  if (!c.copy_stream) {
    EQD_CUDA_OK(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      EQD_CUDA_OK(cudaEventCreateWithFlags(&c.ev_staged[k], cudaEventDisableTiming));
      EQD_CUDA_OK(cudaEventCreateWithFlags(&c.ev_copied[k], cudaEventDisableTiming));
    }
    EQD_CUDA_OK(cudaHostAlloc(reinterpret_cast<void **>(&c.h_err), 2 * sizeof(int), cudaHostAllocDefault));
    c.h_err[0] = c.h_err[1] = 0;
  }
  const int slot = (int)(c.async_issued & 1);
  // the slot's previous read must have reached the host before the slot is reused
  if (c.async_issued - c.async_waited >= 2) {
    EQD_CUDA_OK(cudaEventSynchronize(c.ev_copied[slot]));
    c.async_waited = c.async_issued - 1;
  }
  const size_t need = (size_t)nrows * np + 1;  // rows, then the error word
  if (c.stage_cap[slot] < need) {
    EQD_CUDA_OK(cudaEventSynchronize(c.ev_copied[slot]));
    if (c.d_stage[slot]) cudaFree(c.d_stage[slot]);
    c.d_stage[slot] = nullptr;
    if (cudaMalloc(reinterpret_cast<void **>(&c.d_stage[slot]), need * sizeof(double)) != cudaSuccess)
      return EQD_ERR_OOM;
    c.stage_cap[slot] = need;
  }
  double *st = c.d_stage[slot];
  EQD_CUDA_OK(cudaStreamWaitEvent(c.stream, c.ev_copied[slot], 0));
  for (int r = 0; r < nrows; ++r)
    EQD_CUDA_OK(cudaMemcpyAsync(st + (size_t)r * np, c.fric + (size_t)(rows[r] - 1) * np, np * sizeof(double),
                                cudaMemcpyDeviceToDevice, c.stream));
  int *st_err = reinterpret_cast<int *>(st + (size_t)nrows * np);
  EQD_CUDA_OK(cudaMemcpyAsync(st_err, c.d_err, sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
  EQD_CUDA_OK(cudaEventRecord(c.ev_staged[slot], c.stream));
  EQD_CUDA_OK(cudaStreamWaitEvent(c.copy_stream, c.ev_staged[slot], 0));
  if (np > 0)
    EQD_CUDA_OK(cudaMemcpyAsync(dst, st, (size_t)nrows * np * sizeof(double), cudaMemcpyDeviceToHost, c.copy_stream));
  EQD_CUDA_OK(cudaMemcpyAsync(c.h_err + slot, st_err, sizeof(int), cudaMemcpyDeviceToHost, c.copy_stream));
  EQD_CUDA_OK(cudaEventRecord(c.ev_copied[slot], c.copy_stream));
  *ticket = c.async_issued++;
  return EQD_OK;
}

namespace {
void drop_graph(Context &c) {  // a captured graph holds the kernels' arguments by value
  if (c.graph) {
    cudaGraphExecDestroy(c.graph);
    c.graph = nullptr;
  }
}
}  // namespace

int eqd_gpu_output_setup(eqd_context *X, const int32_t *surface_nodes, int32_t n_surface, int32_t every,
                         int32_t ring_frames) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  if (n_surface < 0 || every < 1 || ring_frames < 1 || (n_surface > 0 && !surface_nodes)) return EQD_ERR_INPUT;
  if (c.out_frames) return EQD_ERR_STATE;  // once per context
  std::vector<int> surf(n_surface);
  for (int k = 0; k < n_surface; ++k) {
    const int j = surface_nodes[k];
    if (j < 1 || j > (int)X->node_dev.size() || X->node_dev[j - 1] < 0) return EQD_ERR_INPUT;
    surf[k] = X->node_dev[j - 1];
  }
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  const size_t len = 3 * (size_t)n_surface + c.npair;
  if (n_surface > 0) RC(dupload(c, c.out_surf, surf));
  RC(dalloc(c, c.out_frames, std::max<size_t>(len, 1) * ring_frames));
  RC(dalloc(c, c.out_count, 1));
  EQD_CUDA_OK(cudaMemset(c.out_count, 0, sizeof(int)));
  c.out_nsurf = n_surface;
  c.out_every = every;
  c.out_ring = ring_frames;
  c.out_drained = 0;
  drop_graph(c);  // the capture joins the step graph
  return EQD_OK;
}

int eqd_gpu_output_drain(eqd_context *X, double *gm, double *src_evol, int32_t max_frames, int32_t *frames,
                         int32_t *first_step) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  if (!c.out_frames) return EQD_ERR_STATE;
  if (max_frames < 0 || !frames || !first_step) return EQD_ERR_INPUT;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  int total = 0;
  EQD_CUDA_OK(cudaMemcpy(&total, c.out_count, sizeof(int), cudaMemcpyDeviceToHost));
  // frames older than the ring were overwritten: hand over the oldest still held
  if (total - c.out_drained > c.out_ring) c.out_drained = total - c.out_ring;
  const int n = (int)std::min<int64_t>(total - c.out_drained, max_frames);
  const size_t len = 3 * (size_t)c.out_nsurf + c.npair;
  for (int k = 0; k < n; ++k) {
    const double *fr = c.out_frames + (size_t)((c.out_drained + k) % c.out_ring) * len;
    if (gm && c.out_nsurf > 0)
      EQD_CUDA_OK(cudaMemcpy(gm + (size_t)k * 3 * c.out_nsurf, fr, 3 * (size_t)c.out_nsurf * sizeof(double),
                             cudaMemcpyDeviceToHost));
    if (src_evol && c.npair > 0)
      EQD_CUDA_OK(cudaMemcpy(src_evol + (size_t)k * c.npair, fr + 3 * (size_t)c.out_nsurf,
                             (size_t)c.npair * sizeof(double), cudaMemcpyDeviceToHost));
  }
  *frames = n;
  *first_step = (int32_t)(c.out_drained * c.out_every + 1);
  c.out_drained += n;
  return EQD_OK;
}

int eqd_gpu_fetch_wait(eqd_context *X, int64_t ticket) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  if (ticket < 0 || ticket >= c.async_issued || ticket < c.async_issued - 2) return EQD_ERR_INPUT;
  cudaSetDevice(c.device);
  const int slot = (int)(ticket & 1);
  EQD_CUDA_OK(cudaEventSynchronize(c.ev_copied[slot]));
  if (ticket + 1 > c.async_waited) c.async_waited = ticket + 1;
  return err_status(c.h_err[slot]);
}

int eqd_gpu_fetch_fault(eqd_context *X, double *fric, double *fnft) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  const int np = c.npair;
  if (np == 0) return EQD_OK;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  std::vector<double> fr(100 * (size_t)np);
  if (fric) {
    EQD_CUDA_OK(cudaMemcpy(fr.data(), c.fric, fr.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int i = 0; i < np; ++i)
      for (int k = 0; k < 100; ++k) fric[100 * (size_t)i + k] = fr[k * (size_t)np + i];
  }
  if (fnft) EQD_CUDA_OK(cudaMemcpy(fnft, c.fnft, np * sizeof(double), cudaMemcpyDeviceToHost));
  return EQD_OK;
}

int eqd_gpu_fetch_fric_rows(eqd_context *X, const int32_t *rows, int32_t nrows, double *dst) {
  if (!X) return EQD_ERR_STATE;
  if (nrows < 0 || (nrows > 0 && (!rows || !dst))) return EQD_ERR_INPUT;
  Context &c = X->c;
  const int np = c.npair;
  for (int r = 0; r < nrows; ++r)
    if (rows[r] < 1 || rows[r] > 100) return EQD_ERR_INPUT;
  if (np == 0 || nrows == 0) return EQD_OK;
  cudaSetDevice(c.device);
  for (int r = 0; r < nrows; ++r)
    EQD_CUDA_OK(cudaMemcpyAsync(dst + (size_t)r * np, c.fric + (size_t)(rows[r] - 1) * np, np * sizeof(double),
                                cudaMemcpyDeviceToHost, c.stream));
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  return EQD_OK;
}

void *eqd_host_alloc(int64_t bytes) {
  void *p = nullptr;
  if (bytes <= 0 || cudaHostAlloc(&p, (size_t)bytes, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

int eqd_host_free(void *p) {
  if (p && cudaFreeHost(p) != cudaSuccess) return EQD_ERR_CUDA;
  return EQD_OK;
}

int eqd_gpu_fetch(eqd_context *X, eqd_host_arrays *a) {
  if (!X || !a) return EQD_ERR_STATE;
  Context &c = X->c;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  if (a->nnode != X->nnode_mesh || a->nelem != c.nelem) return EQD_ERR_INPUT;
  const int nn = c.nnode, np_ = c.npml;
  Scratch<double> vel(3 * (size_t)nn), disp(3 * (size_t)nn), F(3 * (size_t)nn), im(nn);  // copied into
  Scratch<double> v9(9 * (size_t)np_), vh(3 * (size_t)np_), F9(9 * (size_t)np_);  // (no serial zero fill)
  EQD_CUDA_OK(cudaMemcpy(vel.data(), c.vel, vel.size() * 8, cudaMemcpyDeviceToHost));
  EQD_CUDA_OK(cudaMemcpy(disp.data(), c.disp, disp.size() * 8, cudaMemcpyDeviceToHost));
  EQD_CUDA_OK(cudaMemcpy(im.data(), c.inv_mass, im.size() * 8, cudaMemcpyDeviceToHost));
  auto get32 = [&](auto &dst, const float *src) -> int {
    Scratch<float> t(dst.size());
    if (!t.empty() && cudaMemcpy(t.data(), src, t.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return EQD_ERR_CUDA;
    const long long nt = (long long)t.size();
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < nt; ++q) dst[q] = t[q];
    return EQD_OK;
  };
  if (c.fp32) {
    RC(get32(F, c.F32));
    if (c.npair > 0) {
      std::vector<double> fs(3 * (size_t)2 * c.npair);
      std::vector<int> ps(c.npair), pm(c.npair);
      EQD_CUDA_OK(cudaMemcpy(fs.data(), c.Fsplit, fs.size() * 8, cudaMemcpyDeviceToHost));
      EQD_CUDA_OK(cudaMemcpy(ps.data(), c.pair_s, ps.size() * 4, cudaMemcpyDeviceToHost));
      EQD_CUDA_OK(cudaMemcpy(pm.data(), c.pair_m, pm.size() * 4, cudaMemcpyDeviceToHost));
      for (int i = 0; i < c.npair; ++i)
        for (int q = 0; q < 3; ++q) {
          F[(size_t)q * nn + ps[i]] = fs[(size_t)q * 2 * c.npair + 2 * i];
          F[(size_t)q * nn + pm[i]] = fs[(size_t)q * 2 * c.npair + 2 * i + 1];
        }
    }
  } else {
    EQD_CUDA_OK(cudaMemcpy(F.data(), c.F, F.size() * 8, cudaMemcpyDeviceToHost));
  }
  if (np_ > 0) {
    EQD_CUDA_OK(cudaMemcpy(vh.data(), c.vh, vh.size() * 8, cudaMemcpyDeviceToHost));
    if (c.fp32) {
      RC(get32(v9, c.v9_32));
      RC(get32(F9, c.F9_32));
    } else {
      EQD_CUDA_OK(cudaMemcpy(v9.data(), c.v9, v9.size() * 8, cudaMemcpyDeviceToHost));
      EQD_CUDA_OK(cudaMemcpy(F9.data(), c.F9, F9.size() * 8, cudaMemcpyDeviceToHost));
    }
  }
  auto eq = [&](int j, int k) { return a->eqNumIndexArr[a->eqNumStartIndexLoc[j] + k - 1]; };
  // every device node d writes only the entries of its own Fortran node j
#pragma omp parallel for schedule(static)
  for (int d = 0; d < nn; ++d) {
    const int j = X->node_orig[d];
    if (j < 0) continue;  // padding
    for (int k = 0; k < 3; ++k) {
      if (a->velArr) a->velArr[3 * (size_t)j + k] = vel[k * (size_t)nn + d];
      if (a->dispArr) a->dispArr[3 * (size_t)j + k] = disp[k * (size_t)nn + d];
    }
    const double sc = c.f_is_acc ? 1.0 : im[d];
    if (d < c.n_int) {
      for (int k = 1; k <= 3; ++k) {
        const int e = eq(j, k);
        if (a->v1) a->v1[e - 1] = vel[(k - 1) * (size_t)nn + d];
        if (a->nodalForceArr) a->nodalForceArr[e - 1] = F[(k - 1) * (size_t)nn + d] * sc;
      }
    } else if (im[d] != 0.0) {
      const int p = d - c.n_int;
      for (int k = 1; k <= 12; ++k) {
        const int e = eq(j, k);
        const double v = k <= 9 ? v9[(k - 1) * (size_t)np_ + p] : vh[(k - 10) * (size_t)np_ + p];
        const double f = k <= 9 ? F9[(k - 1) * (size_t)np_ + p] : F[(k - 10) * (size_t)nn + d];
        if (a->v1) a->v1[e - 1] = v;
        if (a->nodalForceArr) a->nodalForceArr[e - 1] = f * sc;
      }
    }
  }
  // element state
  if (a->stressArr) {
    for (int grp = 0; grp < 2; ++grp) {
      const std::vector<int> &ids = grp == 0 ? X->gi_orig : X->gp_orig;
      const int m = (int)ids.size();
      if (m == 0) continue;
      const int nstress = grp == 0 ? (c.sc.C_Q != 0 ? 12 : 6) : 15;
      // stress component q of device slot i at src[q * ld + i], into the element's stressArr entries
      auto scatter = [&](const auto *src, size_t ld) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < m; ++i) {
          if (ids[i] < 0) continue;  // empty slot of the binary32 tiles
          const int64_t base = a->stressCompIndexArr[ids[i]];
          for (int q = 0; q < nstress; ++q) a->stressArr[base + q] = (double)src[q * ld + i];
        }
      };
      if (c.fp32) {
        const ElemGroup<float> &g = grp == 0 ? c.gi32 : c.gp32;
        Scratch<float> s32(nstress * (size_t)g.ld);
        EQD_CUDA_OK(cudaMemcpy(s32.data(), g.stress, s32.size() * 4, cudaMemcpyDeviceToHost));
        scatter(s32.data(), (size_t)g.ld);
      } else {
        const ElemGroup<double> &g = grp == 0 ? c.gi64 : c.gp64;
        Scratch<double> st(nstress * (size_t)m);
        EQD_CUDA_OK(cudaMemcpy(st.data(), g.stress, st.size() * 8, cudaMemcpyDeviceToHost));
        scatter(st.data(), (size_t)m);
      }
    }
  }
  const double *dps = c.fp32 ? c.gi32.pstrain : c.gi64.pstrain;
  const int nps = c.fp32 ? c.gi32.ne : c.gi64.ne;
  if (a->pstrain && dps) {
    Scratch<double> ps(nps);
    EQD_CUDA_OK(cudaMemcpy(ps.data(), dps, ps.size() * 8, cudaMemcpyDeviceToHost));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nps; ++i)
      if (X->gi_orig[i] >= 0) a->pstrain[X->gi_orig[i]] = ps[i];
  }
  RC(eqd_gpu_fetch_fault(X, a->fric, a->fnft));
  if (c.nstep > 0) {
    const int ncol = a->numOnFaultSt > 0 ? a->numOnFaultSt : 1;
    if (a->onFaultQuantHistSCECForm && c.onhist)
      EQD_CUDA_OK(cudaMemcpy(a->onFaultQuantHistSCECForm, c.onhist, 12 * (size_t)c.nstep * ncol * 8, cudaMemcpyDeviceToHost));
    if (a->OffFaultStGramSCEC && c.offhist)
      EQD_CUDA_OK(cudaMemcpy(a->OffFaultStGramSCEC, c.offhist, (size_t)(c.nOffRows + 1) * c.nstep * 8, cudaMemcpyDeviceToHost));
    if (a->onFaultTPHist && c.tp_hist) {
      std::vector<double> h(2 * (size_t)c.npair * c.nstep);
      EQD_CUDA_OK(cudaMemcpy(h.data(), c.tp_hist, h.size() * 8, cudaMemcpyDeviceToHost));
      for (int t = 0; t < c.nstep; ++t)
        for (int i = 0; i < c.npair; ++i)
          for (int k = 0; k < 2; ++k)
            a->onFaultTPHist[2 * ((size_t)i + (size_t)X->nftmx * t) + k] = h[2 * ((size_t)i + (size_t)c.npair * t) + k];
    }
  }
  return EQD_OK;
}

int eqd_gpu_finalize(eqd_context *X) {
  if (!X) return EQD_OK;
  Context &c = X->c;
  cudaSetDevice(c.device);
  if (c.stream) cudaStreamSynchronize(c.stream);
  if (c.graph) cudaGraphExecDestroy(c.graph);
  for (cudaEvent_t e : c.prof_events) cudaEventDestroy(e);
  if (c.copy_stream) {
    cudaStreamSynchronize(c.copy_stream);
    cudaStreamDestroy(c.copy_stream);
  }
  if (c.side) {
    cudaStreamSynchronize(c.side);
    cudaStreamDestroy(c.side);
  }
  if (c.ev_fork) cudaEventDestroy(c.ev_fork);
  if (c.ev_join) cudaEventDestroy(c.ev_join);
  for (int k = 0; k < 2; ++k)
    if (c.call_ev[k]) cudaEventDestroy(c.call_ev[k]);
  for (int k = 0; k < 2; ++k) {
    if (c.ev_staged[k]) cudaEventDestroy(c.ev_staged[k]);
    if (c.ev_copied[k]) cudaEventDestroy(c.ev_copied[k]);
    if (c.d_stage[k]) cudaFree(c.d_stage[k]);
  }
  if (c.h_err) cudaFreeHost(c.h_err);
  mlp_free(c);
  for (void *p : c.allocs) cudaFree(p);
  if (c.stream) cudaStreamDestroy(c.stream);
  delete X;
  return EQD_OK;
}

int eqd_gpu_stats(eqd_context *X, int64_t *newton_iters, int64_t *newton_maxhits, int64_t *elem_updates,
                  int64_t *kernel_launches) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  unsigned long long st[4] = {0, 0, 0, 0};
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  EQD_CUDA_OK(cudaMemcpy(st, c.d_stats, sizeof(st), cudaMemcpyDeviceToHost));
  if (newton_iters) *newton_iters = (int64_t)st[0];
  if (newton_maxhits) *newton_maxhits = (int64_t)st[1];
  if (elem_updates) *elem_updates = c.elem_updates;
  if (kernel_launches) *kernel_launches = c.launches_last;
  return EQD_OK;
}

double eqd_gpu_time(eqd_context *X) { return X ? X->c.time : 0.0; }

int eqd_gpu_profile(eqd_context *X, int32_t enable) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  if (enable == 2) {
    for (int k = 0; k < 5; ++k) c.prof_ms[k] = 0.0, c.prof_launches[k] = 0;
    return EQD_OK;
  }
  if (enable == 3) {
    cudaSetDevice(c.device);
    for (int k = 0; k < 2; ++k)
      if (!c.call_ev[k]) EQD_CUDA_OK(cudaEventCreate(&c.call_ev[k]));
    c.profile = 0;
    c.time_calls = 1;
    return EQD_OK;
  }
  if (enable < 0 || enable > 3) return EQD_ERR_INPUT;
  c.profile = enable ? 1 : 0;
  c.time_calls = 0;
  return EQD_OK;
}

int eqd_gpu_kernel_time(eqd_context *X, int32_t kind, double *ms, int64_t *launches) {
  if (!X) return EQD_ERR_STATE;
  if (kind < 0 || kind > 4) return EQD_ERR_INPUT;
  if (ms) *ms = X->c.prof_ms[kind];
  if (launches) *launches = X->c.prof_launches[kind];
  return EQD_OK;
}

int eqd_gpu_newton_log(eqd_context *X, int32_t nsteps, int32_t stride) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  drop_graph(c);
  return newton_log_start(c, nsteps, stride);
}

int eqd_gpu_newton_records(eqd_context *X, double *host, int64_t cap, int64_t *count) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  long long n = 0;
  const int rc = newton_records(c, host, cap, &n);
  if (count) *count = n;
  return rc;
}

int eqd_gpu_mlp_train(eqd_context *X, const eqd_mlp_train_options *opt, float *epoch_loss, float *holdout_loss) {
  if (!X) return EQD_ERR_STATE;
  if (!opt) return EQD_ERR_INPUT;
  Context &c = X->c;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  drop_graph(c);
  RC(mlp_train(c, *opt, epoch_loss, holdout_loss));
  c.mlp_on = 1;
  return EQD_OK;
}

int eqd_gpu_mlp_get(eqd_context *X, float *params, float *norm) {
  if (!X) return EQD_ERR_STATE;
  cudaSetDevice(X->c.device);
  return mlp_get(X->c, params, norm);
}

int eqd_gpu_mlp_set(eqd_context *X, const float *params, const float *norm) {
  if (!X) return EQD_ERR_STATE;
  if (!params || !norm) return EQD_ERR_INPUT;
  Context &c = X->c;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  drop_graph(c);
  RC(mlp_set(c, params, norm));
  c.mlp_on = 1;
  return EQD_OK;
}

int eqd_gpu_mlp_enable(eqd_context *X, int32_t on) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  if (on && !c.mlp) return EQD_ERR_STATE;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  drop_graph(c);
  c.mlp_on = on ? 1 : 0;
  return EQD_OK;
}

int eqd_gpu_newton_replay(eqd_context *X, int32_t learned, int32_t fast, int64_t counts[5], double *v_host) {
  if (!X) return EQD_ERR_STATE;
  if (!counts) return EQD_ERR_INPUT;
  Context &c = X->c;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  long long cc[5] = {0, 0, 0, 0, 0};
  RC(newton_replay(c, learned, fast, cc, v_host));
  for (int k = 0; k < 5; ++k) counts[k] = cc[k];
  return EQD_OK;
}

int eqd_gpu_newton_replay_records(eqd_context *X, int32_t learned, int32_t fast, double *v_host, double *step_host,
                                  int32_t *flags_host) {
  if (!X) return EQD_ERR_STATE;
  Context &c = X->c;
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  long long cc[5] = {0, 0, 0, 0, 0};
  static_assert(sizeof(int32_t) == sizeof(int), "flags are 32-bit");
  return newton_replay(c, learned, fast, cc, v_host, step_host, reinterpret_cast<int *>(flags_host));
}

// ---- ensembles ---------------------------------------------------------------------------------
struct eqd_ensemble {
  std::vector<eqd_context *> members;
  std::vector<Context *> ctx;
  int device = 0;
  cudaStream_t stream = nullptr;
  void *nf = nullptr;  // node / fault argument tables
  void *eb = nullptr;  // element argument tables
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  double last_ms = 0.0;
  int mode = 0;              // 0 batched launches in step graphs, 1 one persistent launch per call
  unsigned *bar = nullptr;   // grid-barrier words of the persistent launch
};

namespace {
int ensemble_refresh(eqd_ensemble &E) {
  EQD_CUDA_OK(cudaStreamSynchronize(E.stream));  // no launch reads the tables while they change
  RC(node_fault_batch_update(&E.nf, E.ctx.data(), (int)E.ctx.size()));
  std::vector<ElemConst> k(E.ctx.size());
  for (size_t i = 0; i < E.ctx.size(); ++i) k[i] = make_elem_const(*E.ctx[i]);
  return elem_batch_update(&E.eb, E.ctx.data(), (int)E.ctx.size(), k.data());
}

int ensemble_launch_step(eqd_ensemble &E) {
  RC(launch_node_update_batched(E.nf, E.stream));
  RC(launch_elements_batched(E.eb, E.stream, 2));
  return launch_fault_batched(E.nf, E.stream);
}
}  // namespace

int eqd_ensemble_create(eqd_context *const *members, int32_t n, eqd_ensemble **out) {
  if (!members || n <= 0 || !out) return EQD_ERR_INPUT;
  auto *E = new eqd_ensemble();
  for (int i = 0; i < n; ++i) {
    if (!members[i] || members[i]->c.device != members[0]->c.device) {
      delete E;
      return EQD_ERR_INPUT;
    }
    E->members.push_back(members[i]);
    E->ctx.push_back(&members[i]->c);
  }
  E->device = members[0]->c.device;
  cudaSetDevice(E->device);
  int rc = EQD_OK;
  if (cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&E->ev[0]) != cudaSuccess || cudaEventCreate(&E->ev[1]) != cudaSuccess)
    rc = EQD_ERR_CUDA;
  if (!rc) {
    for (auto *X : E->members) cudaStreamSynchronize(X->c.stream);
    rc = ensemble_refresh(*E);
  }
  if (rc) {
    eqd_ensemble_destroy(E);
    return rc;
  }
  *out = E;
  return EQD_OK;
}

int eqd_ensemble_step(eqd_ensemble *E, int32_t nsteps) {
  if (!E) return EQD_ERR_STATE;
  if (nsteps < 0) return EQD_ERR_INPUT;
  if (nsteps == 0) return EQD_OK;
  cudaSetDevice(E->device);
  for (auto *X : E->members) RC(ensure_times(*X, X->c.nt + nsteps));
  RC(ensemble_refresh(*E));
  int done = 0;
  bool first = false;
  for (auto *c : E->ctx) first |= c->f_is_acc != 0;
  double first_ms = 0.0;
  EQD_CUDA_OK(cudaEventRecord(E->ev[0], E->stream));
  if (first) {  // members fresh from init consume their stored acceleration in this step
    RC(ensemble_launch_step(*E));
    EQD_CUDA_OK(cudaEventRecord(E->ev[1], E->stream));
    for (auto *c : E->ctx) c->f_is_acc = 0;
    RC(ensemble_refresh(*E));
    float ms = 0.f;
    EQD_CUDA_OK(cudaEventElapsedTime(&ms, E->ev[0], E->ev[1]));
    first_ms = ms;
    EQD_CUDA_OK(cudaEventRecord(E->ev[0], E->stream));
    ++done;
  }
  if (E->mode == 1 && nsteps > done) {  // every remaining step in one cooperative launch
    RC(launch_ensemble_persistent(E->nf, E->eb, nsteps - done, E->bar, E->ctx[0]->d_err, E->stream));
    done = nsteps;
  }
  if (nsteps - done >= kGraphSteps) {
    if (!E->graph) {
      cudaGraph_t g;
      EQD_CUDA_OK(cudaStreamBeginCapture(E->stream, cudaStreamCaptureModeThreadLocal));
      int rc = EQD_OK;
      for (int k = 0; k < kGraphSteps && !rc; ++k) rc = ensemble_launch_step(*E);
      const cudaError_t e = cudaStreamEndCapture(E->stream, &g);
      if (rc) return rc;
      EQD_CUDA_OK(e);
      const cudaError_t ei = cudaGraphInstantiate(&E->graph, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) {
        E->graph = nullptr;
        return EQD_ERR_CUDA;
      }
    }
    while (nsteps - done >= kGraphSteps) {
      EQD_CUDA_OK(cudaGraphLaunch(E->graph, E->stream));
      done += kGraphSteps;
    }
  }
  for (; done < nsteps; ++done) RC(ensemble_launch_step(*E));
  EQD_CUDA_OK(cudaEventRecord(E->ev[1], E->stream));
  EQD_CUDA_OK(cudaStreamSynchronize(E->stream));
  {
    float ms = 0.f;
    EQD_CUDA_OK(cudaEventElapsedTime(&ms, E->ev[0], E->ev[1]));
    E->last_ms = first_ms + ms;
  }
  EQD_CUDA_OK(cudaGetLastError());
  int status = EQD_OK;
  for (auto *X : E->members) {
    Context &c = X->c;
    int err = 0;
    EQD_CUDA_OK(cudaMemcpy(&err, c.d_err, sizeof(int), cudaMemcpyDeviceToHost));
    c.nt += nsteps;
    c.time = X->times[c.nt];
    c.elem_updates += (int64_t)c.nelem * nsteps;
    if (err & 2) status = EQD_ERR_TIMEOUT;
    else if (err && !status) status = EQD_ERR_NAN;
  }
  return status;
}

int eqd_ensemble_destroy(eqd_ensemble *E) {
  if (!E) return EQD_OK;
  cudaSetDevice(E->device);
  if (E->stream) cudaStreamSynchronize(E->stream);
  if (E->graph) cudaGraphExecDestroy(E->graph);
  for (auto &e : E->ev)
    if (e) cudaEventDestroy(e);
  node_fault_batch_free(E->nf);
  elem_batch_free(E->eb);
  if (E->bar) cudaFree(E->bar);
  if (E->stream) cudaStreamDestroy(E->stream);
  delete E;
  return EQD_OK;
}

int eqd_ensemble_mode(eqd_ensemble *E, int32_t mode) {
  if (!E) return EQD_ERR_STATE;
  if (mode != 0 && mode != 1) return EQD_ERR_INPUT;
  if (mode == 1) {
    for (auto *c : E->ctx)
      if (c->sc.friclaw > 2 || c->sc.C_Q != 0 || ((c->sc.rdampm != 0.0) && c->sc.C_elastic != 0))
        return EQD_ERR_UNSUPPORTED;
    cudaSetDevice(E->device);
    if (!E->bar && cudaMalloc(&E->bar, 2 * sizeof(unsigned)) != cudaSuccess) {
      cudaGetLastError();
      E->bar = nullptr;
      return EQD_ERR_OOM;
    }
    int coop = 0;
    EQD_CUDA_OK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, E->device));
    if (!coop) return EQD_ERR_UNSUPPORTED;
  }
  E->mode = mode;
  return EQD_OK;
}

int eqd_ensemble_time(eqd_ensemble *E, double *ms) {
  if (!E) return EQD_ERR_STATE;
  if (!ms) return EQD_ERR_INPUT;
  *ms = E->last_ms;
  return EQD_OK;
}

int eqd_gpu_newton_counts(eqd_context *X, int64_t out[5]) {
  if (!X) return EQD_ERR_STATE;
  if (!out) return EQD_ERR_INPUT;
  Context &c = X->c;
  unsigned long long st[5] = {0, 0, 0, 0, 0};
  cudaSetDevice(c.device);
  EQD_CUDA_OK(cudaStreamSynchronize(c.stream));
  EQD_CUDA_OK(cudaMemcpy(st, c.d_stats, sizeof(st), cudaMemcpyDeviceToHost));
  for (int k = 0; k < 5; ++k) out[k] = (int64_t)st[k];
  return EQD_OK;
}

int eqd_gpu_init_times(eqd_context *X, double ms[8]) {
  if (!X) return EQD_ERR_STATE;
  if (!ms) return EQD_ERR_INPUT;
  for (int k = 0; k < 8; ++k) ms[k] = X->init_ms[k];
  return EQD_OK;
}

int eqd_gpu_table_info(eqd_context *X, int32_t group, int64_t info[8]) {
  if (!X) return EQD_ERR_STATE;
  if ((group != 0 && group != 1) || !info) return EQD_ERR_INPUT;
  const Context &c = X->c;
  const ElemGroup<float> &g = group == 0 ? c.gi32 : c.gp32;
  info[0] = (!c.fp32 || g.ne == 0) ? 0 : (g.nrec > 0 ? 2 : 1);
  info[1] = c.fp32 ? g.ne_live : (group == 0 ? c.gi64.ne : c.gp64.ne);
  info[2] = g.nrec;
  info[3] = g.rec_len;
  info[4] = c.fp32 ? g.ntiles : 0;
  info[5] = c.fp32 ? (int64_t)g.ntiles * g.tile : 0;
  info[6] = c.fp32 ? g.max_tile_nodes : 0;
  info[7] = c.fp32 ? g.sum_tile_nodes : 0;
  return EQD_OK;
}

int eqd_gpu_fp64_fma_peak(int32_t device, double *tflops) {
  if (!tflops) return EQD_ERR_INPUT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return EQD_ERR_NO_DEVICE;
  }
  EQD_CUDA_OK(cudaSetDevice(device));
  cudaDeviceProp prop;
  EQD_CUDA_OK(cudaGetDeviceProperties(&prop, device));
  double *out = nullptr;
  EQD_CUDA_OK(cudaMalloc(&out, sizeof(double)));
  const int threads = 256, blocks = prop.multiProcessorCount * 8, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp64_fma_chain<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  fp64_fma_chain<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return EQD_ERR_CUDA;
  *tflops = 2.0 * 8.0 * (double)iters * threads * blocks / (ms * 1e-3) / 1e12;
  return EQD_OK;
}

int eqd_host_element_order(const eqd_host_arrays *a, int32_t group, int32_t tile_shape, int32_t *out,
                           int64_t cap, int64_t *n_out, double *live) {
  if (!a || !n_out || (group != 0 && group != 1) || a->nelem < 0 || !a->elemTypeArr ||
      !a->nodeElemIdRelation || !a->meshCoor || a->nnode <= 0)
    return EQD_ERR_INPUT;
  if (!connectivity_in_range(*a)) return EQD_ERR_INPUT;
  std::vector<int> ids;
  for (int e = 0; e < a->nelem; ++e) {
    const int t = a->elemTypeArr[e];
    if (group == 0 ? (t == 1 || t > 10) : (t == 2)) ids.push_back(e);
  }
  const int ts = tile_shape > 0 ? tile_shape : (4 | 8 << 8 | 4 << 16);
  const int bx = ts & 255, by = (ts >> 8) & 255, bz = (ts >> 16) & 255;
  if (bx < 1 || by < 1 || bz < 1) return EQD_ERR_INPUT;
  const double f = brick_order(*a, ids, bx, bz, by, eqd::tile_size_interior());
  if (live) *live = f;
  *n_out = (int64_t)ids.size();
  if (!out || cap < (int64_t)ids.size()) return out ? EQD_ERR_INPUT : EQD_OK;
  std::copy(ids.begin(), ids.end(), out);
  return EQD_OK;
}

int eqd_host_node_order(const eqd_host_arrays *a, int32_t *out, int64_t cap, int64_t *n_out, int32_t counts[4]) {
  if (!a || !n_out || !counts) return EQD_ERR_INPUT;
  NodeOrder o;
  const int rc = device_node_order(*a, o);
  if (rc) return rc;
  counts[0] = o.n_split;
  counts[1] = o.n_int;
  counts[2] = o.npml_live;
  counts[3] = (int32_t)o.orig.size();
  *n_out = (int64_t)o.orig.size();
  if (!out || cap < (int64_t)o.orig.size()) return out ? EQD_ERR_INPUT : EQD_OK;
  std::copy(o.orig.begin(), o.orig.end(), out);
  return EQD_OK;
}

}  // extern "C"
