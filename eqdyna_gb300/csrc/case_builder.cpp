// Host-side case setup: restates the part of the EQdyna Fortran program that runs before the
// time loop, producing the globalvar arrays (Fortran layout, 1-based index values) that the
// GPU hot path and the oracle consume.  Single process only (npx = npy = npz = 1), which is the
// configuration in which the reference's MPI halo sums are no-ops
// (src/assembleGlobalMass.f90:89).
//
// Followed routines (reference file:line):
//   b-file readers ............ src/readInputFiles.f90:2-312
//   grid lines ................ src/meshgen.f90:447-560 (getLocalOneDimCoorArrAndSize)
//   node/element loops ........ src/meshgen.f90:64-107, helpers :562-996
//   wedges .................... src/library_degeneration.f90:3-97
//   fault areas ............... src/meshgen.f90:113-155
//   on-fault fields ........... src/netcdf_io.f90:70-106
//   station index rows ........ src/eqdyna3d.f90:153-189 (allocInitAfterMeshGen)
//   shape tables / mass / HG .. src/calcLocalShapeFunc.f90, src/calcGlobalShapeFunc.f90,
//                               src/assembleGlobalMass.f90:12-38,283-406, src/library.f90:60-93
//   initial split-node vel .... src/eqdyna3d.f90:191-212 (init_vel)
#include "eqdyna_case.h"
#include "eqd_geometry.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

thread_local std::string g_case_error;

struct CaseError : std::runtime_error {
  int code;
  CaseError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(const std::string &m, int code = EQD_ERR_INPUT) { throw CaseError(code, m); }

const double kPi = 4.0 * std::atan(1.0);  // pi=4*atan(1.0_dp) (src/globalvar.f90:16)
const double kTol = 1.0e-5;               // tol (src/globalvar.f90:31)
const double kGrav = 9.8;
const int kMaxLine = 1000000;             // np, the loop bound of the stretched grid search

// Fortran NINT / IDNINT: round half away from zero.
inline long fnint(double x) { return std::lround(x); }

// ---------------------------------------------------------------------------------------------
// Fortran list-directed style record reader: every read statement consumes one line.
class Records {
 public:
  explicit Records(const std::string &path) : path_(path) {
    std::ifstream f(path);
    if (!f) fail("missing input file " + path);
    std::string line;
    while (std::getline(f, line)) lines_.push_back(line);
  }
  bool has_more() const { return pos_ < lines_.size(); }
  void skip() {
    if (pos_ >= lines_.size()) fail("unexpected end of " + path_);
    ++pos_;
  }
  std::vector<double> reals(size_t n) {
    std::vector<double> out;
    while (out.size() < n) {
      if (pos_ >= lines_.size()) fail("unexpected end of " + path_);
      std::string s = lines_[pos_++];
      for (char &ch : s)
        if (ch == ',' || ch == '\t') ch = ' ';
      std::istringstream is(s);
      std::string tok;
      while (out.size() < n && (is >> tok)) {
        for (char &ch : tok)
          if (ch == 'd' || ch == 'D') ch = 'e';
        char *end = nullptr;
        double v = std::strtod(tok.c_str(), &end);
        if (end == tok.c_str()) fail("cannot parse '" + tok + "' in " + path_);
        out.push_back(v);
      }
    }
    return out;
  }
  double real() { return reals(1)[0]; }
  int integer() {
    double v = real();
    if (v != std::floor(v)) fail("expected an integer in " + path_);
    return static_cast<int>(v);
  }

 private:
  std::string path_;
  std::vector<std::string> lines_;
  size_t pos_ = 0;
};

// ---------------------------------------------------------------------------------------------
struct Inputs {
  // bGlobal.txt (src/readInputFiles.f90:28-57)
  int mode = 1, C_elastic = 1, C_nuclea = 0;
  double C_degen = 0;
  int insertFaultType = 0, friclaw = 1, ntotft = 1, nucfault = 1, TPV = -1;
  int output_plastic = 0, outputGroundMotion = 0, outputFinalSurfDisp = 0;
  int npx = 1, npy = 1, npz = 1;
  double totalSimuTime = 0, dt = 0;
  int nmat = 1, n2mat = 3;
  double roumax = 0, rhow = 0, gamar = 0, rdampk = 0, vmaxPML = 0;
  double xsource = 0, ysource = 0, zsource = 0, nucR = 0, nucRuptVel = 0, nucdtau0 = 0, nucT = 0;
  double str1ToFaultAngle = 0, devStrToStrVertRatio = 0, bulk = 0, coheplas = 0;
  double fstrike = 0, fdip = 0, slipRateThres = 0;
  // bModelGeometry.txt (src/readInputFiles.f90:87-95)
  double xmin = 0, xmax = 0, ymin = 0, ymax = 0, zmin = 0, zmax = 0;
  int dis4uniF = 0, dis4uniB = 0;
  double rat = 1, dx = 0, dy = 0, dz = 0;
  // bFaultGeometry.txt, one fault
  double fxmin = 0, fxmax = 0, fymin = 0, fymax = 0, fzmin = 0, fzmax = 0;
  // bMaterial.txt: material(i,j) stored row-major [i*n2mat + j]
  std::vector<double> material;
  // bStations.txt
  int nOffSt = 0, nOnSt = 0;
  std::vector<double> xonfs;  // (2, nOnSt) metres
  std::vector<double> x4nds;  // (3, nOffSt) metres
  // bFault_Rough_Geometry.txt
  int nnx = 0, nnz = 0;
  double dxtmp = 0, rough_fx_min = 0, rough_fz_min = 0, rough_fx_max = 0;
  std::vector<double> rough_geo;  // (3, nnx*nnz)
  // on_fault_vars_input.bin
  int ofv_nfx = 0, ofv_nfz = 0;
  std::vector<double> ofv;  // (nfx, nfz, 24)
  // compile-time constants of the reference made runtime switches (bGPU.txt)
  int nPML = 6, C_Q = 0, C_hg = 1;
  double R = 0.01, kapa_hg = 0.1, rdampm = 0.0;
  // extension with no reference counterpart: the initial creep rate along the initial shear
  // traction instead of along strike (src/netcdf_io.f90:98-100 always uses strike), for
  // rate-and-state faults loaded along dip
  int vini_along_shear = 0;
};

double mat_in(const Inputs &in, int i, int j) {  // material(i,j), 1-based
  return in.material[static_cast<size_t>(i - 1) * in.n2mat + (j - 1)];
}

void read_inputs(const std::string &dir, Inputs &in) {
  {
    Records r(dir + "/bGlobal.txt");
    in.mode = r.integer();
    in.C_elastic = r.integer();
    in.C_nuclea = r.integer();
    in.C_degen = r.real();
    in.insertFaultType = r.integer();
    in.friclaw = r.integer();
    in.ntotft = r.integer();
    in.nucfault = r.integer();
    in.TPV = r.integer();
    in.output_plastic = r.integer();
    in.outputGroundMotion = r.integer();
    in.outputFinalSurfDisp = r.integer();
    r.skip();
    auto np3 = r.reals(3);
    in.npx = static_cast<int>(np3[0]);
    in.npy = static_cast<int>(np3[1]);
    in.npz = static_cast<int>(np3[2]);
    r.skip();
    in.totalSimuTime = r.real();
    in.dt = r.real();
    r.skip();
    auto nm = r.reals(2);
    in.nmat = static_cast<int>(nm[0]);
    in.n2mat = static_cast<int>(nm[1]);
    auto rr = r.reals(3);
    in.roumax = rr[0];
    in.rhow = rr[1];
    in.gamar = rr[2];
    auto rv = r.reals(2);
    in.rdampk = rv[0];
    in.vmaxPML = rv[1];
    r.skip();
    auto src = r.reals(3);
    in.xsource = src[0];
    in.ysource = src[1];
    in.zsource = src[2];
    auto nuc = r.reals(4);
    in.nucR = nuc[0];
    in.nucRuptVel = nuc[1];
    in.nucdtau0 = nuc[2];
    in.nucT = nuc[3];
    auto st = r.reals(2);
    in.str1ToFaultAngle = st[0] * kPi / 180.0;  // src/readInputFiles.f90:59
    in.devStrToStrVertRatio = st[1];
    auto bc = r.reals(2);
    in.bulk = bc[0];
    in.coheplas = bc[1];
    auto sd = r.reals(2);
    in.fstrike = sd[0];
    in.fdip = sd[1];
    in.slipRateThres = r.real();
  }
  {
    Records r(dir + "/bModelGeometry.txt");
    auto a = r.reals(2);
    in.xmin = a[0];
    in.xmax = a[1];
    a = r.reals(2);
    in.ymin = a[0];
    in.ymax = a[1];
    a = r.reals(2);
    in.zmin = a[0];
    in.zmax = a[1];
    r.skip();
    a = r.reals(2);
    in.dis4uniF = static_cast<int>(a[0]);
    in.dis4uniB = static_cast<int>(a[1]);
    in.rat = r.real();
    a = r.reals(3);
    in.dx = a[0];
    in.dy = a[1];
    in.dz = a[2];
  }
  if (in.ntotft != 1) fail("only one fault is supported (the reference stops for iFault>1, "
                           "src/meshgen.f90:806)", EQD_ERR_UNSUPPORTED);
  if (in.npx * in.npy * in.npz < 1) fail("bad npx*npy*npz");
  {
    Records r(dir + "/bFaultGeometry.txt");
    r.skip();
    auto a = r.reals(2);
    in.fxmin = a[0];
    in.fxmax = a[1];
    a = r.reals(2);
    in.fymin = a[0];
    in.fymax = a[1];
    a = r.reals(2);
    in.fzmin = a[0];
    in.fzmax = a[1];
  }
  {
    Records r(dir + "/bMaterial.txt");
    for (int i = 0; i < in.nmat; ++i) {
      auto row = r.reals(in.n2mat);
      in.material.insert(in.material.end(), row.begin(), row.end());
    }
  }
  {
    Records r(dir + "/bStations.txt");
    in.nOffSt = r.integer();
    in.nOnSt = r.integer();
    r.skip();
    for (int i = 0; i < in.nOnSt; ++i) {
      auto p = r.reals(2);
      in.xonfs.push_back(p[0] * 1000.0);
      in.xonfs.push_back(p[1] * 1000.0);
    }
    if (in.nOffSt > 0) r.skip();
    for (int i = 0; i < in.nOffSt; ++i) {
      auto p = r.reals(3);
      for (int k = 0; k < 3; ++k) in.x4nds.push_back(p[k] * 1000.0);
    }
  }
  if (in.insertFaultType > 0) {
    Records r(dir + "/bFault_Rough_Geometry.txt");
    auto h = r.reals(3);
    in.nnx = static_cast<int>(fnint(h[0]));
    in.nnz = static_cast<int>(fnint(h[1]));
    h = r.reals(3);
    in.dxtmp = h[0];
    in.rough_fx_min = h[1];
    in.rough_fz_min = h[2];
    in.rough_fx_max = (in.nnx - 1) * in.dxtmp + in.rough_fx_min;
    in.rough_geo.reserve(static_cast<size_t>(3) * in.nnx * in.nnz);
    for (int i = 0; i < in.nnx * in.nnz; ++i) {
      auto p = r.reals(3);
      in.rough_geo.insert(in.rough_geo.end(), p.begin(), p.end());
    }
  }
  {
    std::string p = dir + "/on_fault_vars_input.bin";
    FILE *f = std::fopen(p.c_str(), "rb");
    if (!f) fail("missing input file " + p);
    int32_t hdr[3];
    if (std::fread(hdr, sizeof(int32_t), 3, f) != 3 || hdr[0] != 24 || hdr[1] <= 0 || hdr[2] <= 0) {
      std::fclose(f);
      fail("bad header in " + p);
    }
    in.ofv_nfx = hdr[1];
    in.ofv_nfz = hdr[2];
    size_t n = static_cast<size_t>(24) * hdr[1] * hdr[2];
    in.ofv.resize(n);
    size_t got = std::fread(in.ofv.data(), sizeof(double), n, f);
    std::fclose(f);
    if (got != n) fail("short read in " + p);
  }
  {
    std::ifstream f(dir + "/bGPU.txt");
    std::string key;
    double val;
    while (f >> key >> val) {
      if (key == "nPML") in.nPML = static_cast<int>(val);
      else if (key == "R") in.R = val;
      else if (key == "C_Q") in.C_Q = static_cast<int>(val);
      else if (key == "C_hg") in.C_hg = static_cast<int>(val);
      else if (key == "kapa_hg") in.kapa_hg = val;
      else if (key == "vini_along_shear") in.vini_along_shear = static_cast<int>(val);
      else if (key == "rdampm") in.rdampm = val;
      else fail("unknown key '" + key + "' in bGPU.txt");
    }
  }
  // option compatibility, src/warning.f90:6-19
  if (in.C_elastic == 0 && in.C_Q == 1) fail("Q model can only work with elastic code");
  if (in.C_Q != 0 && in.rat > 1) fail("Q model can only work with uniform element size");
  if (in.C_Q < 0 || in.C_Q > 2) fail("C_Q must be 0, 1 or 2");
  if (in.output_plastic == 1 && in.C_elastic != 0) fail("plastic strain output needs C_elastic == 0");
  if (in.mode == 2) fail("mode 2 (cycle restart from fault.r.nc) is not built", EQD_ERR_UNSUPPORTED);
  if (in.nPML < 1) fail("nPML must be >= 1 (fixed boundary nodes must be PML nodes)");
}

// ---------------------------------------------------------------------------------------------
// Allocator that leaves new elements uninitialised: the large tables are written in parallel
// loops, so that their pages are first touched by the threads that fill them.
template <class T>
struct DefaultInit : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = DefaultInit<U>;
  };
  DefaultInit() = default;
  template <class U>
  DefaultInit(const DefaultInit<U> &) noexcept {}
  template <class U>
  void construct(U *) noexcept {}
  template <class U, class... Args>
  void construct(U *p, Args &&...args) {
    ::new ((void *)p) U(std::forward<Args>(args)...);
  }
};
template <class T>
using Table = std::vector<T, DefaultInit<T>>;

// parallel zero fill (first touch by many threads)
template <class V>
void zero_fill(V &v, size_t n) {
  v.resize(n);
  double *p = v.data();
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < static_cast<int64_t>(n); ++i) p[i] = 0.0;
}

struct Case {
  Inputs in;
  eqd_scalars sc{};
  // grid lines (1-based in the reference; 0-based here)
  std::vector<double> xline, yline, zline;
  int nx = 0, ny = 0, nz = 0, nxuni = 0, nzuni = 0;
  double PMLb[8] = {0};
  double xmin = 0, xmax = 0, ymin = 0, ymax = 0, zmin = 0, zmax = 0;
  // nodes
  std::vector<double> meshCoor;             // (3, nnode)
  std::vector<int32_t> eqNumStartIndexLoc;  // (nnode)
  std::vector<int32_t> numOfDofPerNodeArr;  // (nnode)
  std::vector<int32_t> eqNumIndexArr;       // (size_eqidx)
  int32_t equationNumCount = 0;
  // elements (built element-major, mat transposed at the end)
  std::vector<int32_t> nodeElemIdRelation;  // (8, nelem)
  std::vector<int32_t> elemTypeArr, stressCompIndexArr;
  std::vector<double> matRows;               // [e*5 + k]
  Table<double> mat;                         // (nelem, 5)
  std::vector<double> stressArr;
  int64_t stressDofCount = 0;
  std::vector<double> eleporep, pstrain, nodalMassArr, fnms;
  Table<double> eledet, elemass, eleshp, ss, phi, v1, velArr, dispArr, nodalForceArr;
  // fault
  int32_t nftnd = 0;
  std::vector<int32_t> nsmp;                 // (2, nftnd)
  std::vector<double> un, us, ud;            // (3, nftnd)
  std::vector<double> arn;                   // (nftnd)
  std::vector<double> fric;                  // (100, nftnd)
  std::vector<double> fnft;                  // (nftnd)
  std::vector<int32_t> fltrc;                // (2, nxuni, nzuni)
  int ixfi = 0, izfi = 0, ifs = 0, ifd = 0;
  std::unordered_map<int32_t, int32_t> slave_to_master;
  std::vector<char> station_level;           // (nz): an off-fault station lies at this depth
  double dip_tan = 0.0, dip_norm = 1.0;      // tan(C_degen), (1 + tan^2)^(1/2): the dipping plane
  std::vector<double> layer_depths;          // material(i, 1), i = 1..nmat (layer bottoms)
  bool layer_depths_sorted = false;          // strictly increasing: a layer is found by bisection
  std::vector<int32_t> cell_plane_start;     // (nx + 2): first element of each x-layer of cells
  // stations
  std::vector<int32_t> anonfs;               // (3, nOnFound)
  std::vector<int32_t> offStIndex;           // (2, nOffFound): station i, node id
  std::vector<int> n4yn;
  std::vector<int32_t> idhist;               // (3, 6*nOffFound)
  std::vector<double> onFaultQuantHistSCECForm, OffFaultStGramSCEC, onFaultTPHist;
  int32_t numOnFaultSt = 0, numOffFaultSt = 0;
  int64_t n_phys_elem = 0;
  // insertFaultInterface keeps its last indices between calls (Fortran locals are SAVEd in
  // practice; the branches cover every node away from measure-zero ties)
  int rough_ixx = 1, rough_izz = 1;
  double pfx = 0, pfz = 0, ycoort = 0;
  // element-local scratch shared by the shape-function routines
  double localShapeFunc[4][8];
};

double &coor(Case &c, int node, int k) { return c.meshCoor[3 * static_cast<size_t>(node - 1) + (k - 1)]; }

// src/meshgen.f90:447-560 with one rank per dimension.
void grid_line(Case &c, int dimId, std::vector<double> &line, int &nuni) {
  const Inputs &in = c.in;
  double h, front, back, minC, maxC;
  if (dimId == 1) {
    nuni = static_cast<int>(fnint((in.fxmax - in.fxmin) / in.dx)) + 1;
    h = in.dx; front = in.fxmin; back = in.fxmax; minC = in.xmin; maxC = in.xmax;
  } else if (dimId == 2) {
    nuni = in.dis4uniF + in.dis4uniB + 1;
    h = in.dy; front = -in.dis4uniF * in.dy; back = in.dis4uniB * in.dy; minC = in.ymin; maxC = in.ymax;
  } else {
    nuni = static_cast<int>(fnint((in.fzmax - in.fzmin) / in.dz)) + 1;
    h = in.dz; front = in.fzmin; back = in.fzmax; minC = in.zmin; maxC = in.zmax;
  }
  int i;
  double cc = front, hh = h;
  for (i = 1; i <= kMaxLine; ++i) {
    hh *= in.rat;
    cc -= hh;
    if (cc <= minC) break;
  }
  const int frontEdge = i + in.nPML;
  cc = back;
  hh = h;
  for (i = 1; i <= kMaxLine; ++i) {
    hh *= in.rat;
    cc += hh;
    if (cc >= maxC) break;
  }
  if (dimId == 3) i = -in.nPML;
  const int size = nuni + frontEdge + i + in.nPML;
  std::vector<double> g(static_cast<size_t>(size) + 1, 0.0);  // 1-based
  g[frontEdge + 1] = front;
  hh = h;
  for (int k = frontEdge; k >= 1; --k) {
    hh *= in.rat;
    g[k] = g[k + 1] - hh;
  }
  for (int k = frontEdge + 2; k <= frontEdge + nuni; ++k) g[k] = g[k - 1] + h;
  if (dimId < 3) {
    hh = h;
    for (int k = frontEdge + nuni + 1; k <= size; ++k) {
      hh *= in.rat;
      g[k] = g[k - 1] + hh;
    }
  }
  if (dimId == 1) {
    c.xmin = g[1]; c.xmax = g[size];
    c.PMLb[0] = g[size - in.nPML]; c.PMLb[1] = g[in.nPML + 1]; c.PMLb[5] = g[size] - g[size - 1];
  } else if (dimId == 2) {
    c.ymin = g[1]; c.ymax = g[size];
    c.PMLb[2] = g[size - in.nPML]; c.PMLb[3] = g[in.nPML + 1]; c.PMLb[6] = g[size] - g[size - 1];
  } else {
    c.zmin = g[1]; c.zmax = g[size];
    c.PMLb[4] = g[in.nPML + 1]; c.PMLb[7] = g[2] - g[1];
  }
  line.assign(g.begin() + 1, g.end());
}

// src/meshgen.f90:768-787
bool on_fault(const Case &c, const double p[3]) {
  const Inputs &in = c.in;
  if (!(p[0] >= in.fxmin - kTol && p[0] <= in.fxmax + kTol && p[1] >= in.fymin - kTol &&
        p[1] <= in.fymax + kTol && p[2] >= in.fzmin - kTol && p[2] <= in.fzmax + kTol))
    return false;
  if (in.C_degen == 0.0 && p[1] == 0.0) return true;
  if (in.C_degen > 3.0) {
    const double t = c.dip_tan;
    double d = std::fabs(p[2] + p[1] * t);
    d = d / c.dip_norm;
    if (d < in.dx / 100.0) return true;
  }
  return false;
}

// src/meshgen.f90:921-962
void insert_fault_interface(Case &c, const double p[3]) {
  const Inputs &in = c.in;
  const double fx1 = in.rough_fx_min, fx2 = in.rough_fx_max, fz1 = in.rough_fz_min;
  int &ixx = c.rough_ixx, &izz = c.rough_izz;
  const double x = p[0], z = p[2];
  if (x < fx2 + kTol && x > fx1 - kTol && z > fz1 - kTol) {
    ixx = static_cast<int>(fnint((x - fx1) / in.dx)) + 1;
    izz = static_cast<int>(fnint((z - fz1) / in.dz)) + 1;
  } else if (x < fx1 - kTol && z > fz1 - kTol) {
    ixx = 1;
    izz = static_cast<int>(fnint((z - fz1) / in.dz)) + 1;
  } else if (x > fx2 + kTol && z > fz1 - kTol) {
    ixx = in.nnx;
    izz = static_cast<int>(fnint((z - fz1) / in.dz)) + 1;
  } else if (x < fx2 + kTol && x > fx1 - kTol && z < fz1 - kTol) {
    ixx = static_cast<int>(fnint((x - fx1) / in.dx)) + 1;
    izz = 1;
  } else if (x < fx1 - kTol && z < fz1 - kTol) {
    ixx = 1;
    izz = 1;
  } else if (x > fx2 + kTol && z < fz1 - kTol) {
    ixx = in.nnx;
    izz = 1;
  }
  const long row = static_cast<long>(in.nnz) * (ixx - 1) + izz;  // 1-based
  if (row < 1 || row > static_cast<long>(in.nnx) * in.nnz)
    fail("rough fault geometry index out of range");
  const double peak = in.rough_geo[3 * (row - 1) + 0];
  c.pfx = in.rough_geo[3 * (row - 1) + 1];
  c.pfz = in.rough_geo[3 * (row - 1) + 2];
  const double y = p[1];
  if (y > -kTol) c.ycoort = y * (c.ymax - peak) / c.ymax + peak;
  else if (y < -kTol) c.ycoort = y * (peak - c.ymin) / (-c.ymin) + peak;
}

// src/meshgen.f90:574-658: identify off-fault station nodes.
bool near_line(double s, double node, double lo_line, double hi_line, bool use_lo, bool use_hi) {
  if (std::fabs(node - s) < kTol) return true;
  if (use_lo && s > lo_line && s < node && (node - s) < (s - lo_line)) return true;
  if (use_hi && s > node && s < hi_line && (s - node) < (hi_line - s)) return true;
  return false;
}

void surface_station(Case &c, int ix, int iy, int iz, const double p[3], int nodeId) {
  const Inputs &in = c.in;
  const int nx = c.nx, ny = c.ny;
  if (!(iy > 1 && iy < ny)) return;
  if (!c.station_level[iz - 1]) return;  // no station within kTol of this grid level's depth
  int part;
  if (ix > 1 && ix < nx) part = 1;
  else if (ix == 1) part = 2;
  else if (ix == nx) part = 3;
  else return;
  for (int i = 0; i < in.nOffSt; ++i) {
    if (c.n4yn[i] != 0) continue;
    const double sx = in.x4nds[3 * i], sy = in.x4nds[3 * i + 1], sz = in.x4nds[3 * i + 2];
    if (!(std::fabs(p[2] - sz) < kTol)) continue;
    bool xok;
    if (part == 1)
      xok = near_line(sx, p[0], c.xline[ix - 2], c.xline[ix], true, true);
    else if (part == 2)
      xok = near_line(sx, p[0], 0.0, c.xline[ix], false, true);
    else  // part 3 has no exact-match clause (src/meshgen.f90:640-641)
      xok = (sx > c.xline[ix - 2] && sx < p[0] && (p[0] - sx) < (sx - c.xline[ix - 2]));
    if (!xok) continue;
    if (!near_line(sy, p[1], c.yline[iy - 2], c.yline[iy], true, true)) continue;
    c.n4yn[i] = 1;
    c.offStIndex.push_back(i + 1);
    c.offStIndex.push_back(nodeId);
    ++c.numOffFaultSt;
    break;
  }
}

// src/meshgen.f90:660-699
void set_equation_numbers(Case &c, const double p[3], int ndofNode) {
  for (int d = 0; d < ndofNode; ++d) {
    if (std::fabs(p[0] - c.xmin) < kTol || std::fabs(p[0] - c.xmax) < kTol ||
        std::fabs(p[1] - c.ymin) < kTol || std::fabs(p[1] - c.ymax) < kTol ||
        std::fabs(p[2] - c.zmin) < kTol) {
      c.eqNumIndexArr.push_back(-1);
    } else {
      c.eqNumIndexArr.push_back(++c.equationNumCount);
    }
  }
}

void ensure_node(Case &c, int nodeId) {
  if (static_cast<size_t>(nodeId) > c.eqNumStartIndexLoc.size()) {
    c.eqNumStartIndexLoc.resize(nodeId, 0);
    c.numOfDofPerNodeArr.resize(nodeId, 0);
    c.meshCoor.resize(static_cast<size_t>(3) * nodeId, 0.0);
  }
}

// src/meshgen.f90:789-902 (one fault)
void create_master_node(Case &c, int ix, int iy, int iz, const double p[3], int nodeId) {
  const Inputs &in = c.in;
  (void)iy;
  if (!on_fault(c, p)) return;
  const int k = ++c.nftnd;
  const int msnode = c.nx * c.ny * c.nz + k;
  ensure_node(c, msnode);
  c.nsmp.push_back(nodeId);
  c.nsmp.push_back(msnode);
  c.slave_to_master[nodeId] = msnode;
  c.eqNumStartIndexLoc[msnode - 1] = static_cast<int32_t>(c.eqNumIndexArr.size());
  c.numOfDofPerNodeArr[msnode - 1] = 3;
  coor(c, msnode, 1) = p[0];
  coor(c, msnode, 2) = p[1];
  coor(c, msnode, 3) = p[2];
  if (in.insertFaultType > 0) coor(c, msnode, 2) = c.ycoort;
  for (int d = 0; d < 3; ++d) c.eqNumIndexArr.push_back(++c.equationNumCount);
  // on-fault station
  for (int i = 0; i < in.nOnSt; ++i) {
    if (std::fabs(p[0] - in.xonfs[2 * i]) < kTol && std::fabs(p[2] - in.xonfs[2 * i + 1]) < kTol) {
      c.anonfs.push_back(k);
      c.anonfs.push_back(i + 1);
      c.anonfs.push_back(1);
      ++c.numOnFaultSt;
      break;
    }
  }
  // unit vectors
  const double s = in.fstrike * kPi / 180.0;
  const double d = (in.C_degen > 3.0) ? in.C_degen * kPi / 180.0 : 90.0 * kPi / 180.0;
  double n[3] = {std::cos(s) * std::sin(d), -std::sin(s) * std::sin(d), std::cos(d)};
  double t[3] = {-std::sin(s), -std::cos(s), 0.0};
  double b[3] = {std::cos(s) * std::cos(d), std::sin(s) * std::cos(d), std::sin(d)};
  if (in.insertFaultType > 0) {
    const double pfx = c.pfx, pfz = c.pfz;
    const double qn = std::pow(pfx * pfx + 1.0 + pfz * pfz, 0.5);
    const double qs = std::pow(1.0 + pfx * pfx, 0.5);
    n[0] = -pfx / qn; n[1] = 1.0 / qn; n[2] = -pfz / qn;
    t[0] = 1.0 / qs; t[1] = pfx / qs; t[2] = 0.0;
    b[0] = t[1] * n[2] - t[2] * n[1];
    b[1] = t[2] * n[0] - t[0] * n[2];
    b[2] = t[0] * n[1] - t[1] * n[0];
  }
  for (int q = 0; q < 3; ++q) {
    c.un.push_back(n[q]);
    c.us.push_back(t[q]);
    c.ud.push_back(b[q]);
  }
  // area bookkeeping
  if (c.ixfi == 0) c.ixfi = ix;
  if (c.izfi == 0) c.izfi = iz;
  c.ifs = ix - c.ixfi + 1;
  c.ifd = iz - c.izfi + 1;
  if (c.ifs < 1 || c.ifs > c.nxuni || c.ifd < 1 || c.ifd > c.nzuni)
    fail("fault node outside the uniform fault grid");
  const size_t slot = 2 * (static_cast<size_t>(c.ifs - 1) + static_cast<size_t>(c.nxuni) * (c.ifd - 1));
  c.fltrc[slot] = msnode;
  c.fltrc[slot + 1] = k;
}

// src/meshgen.f90:161-207
void set_material(Case &c, int e, const double ctr[3]) {
  const Inputs &in = c.in;
  double *m = &c.matRows[5 * static_cast<size_t>(e - 1)];
  if (in.nmat == 1 && in.n2mat == 3) {
    m[0] = mat_in(in, 1, 1); m[1] = mat_in(in, 1, 2); m[2] = mat_in(in, 1, 3);
  } else if (in.nmat > 1 && in.n2mat == 4) {
    const double az = std::fabs(ctr[2]);
    if (az < mat_in(in, 1, 1)) {
      m[0] = mat_in(in, 1, 2); m[1] = mat_in(in, 1, 3); m[2] = mat_in(in, 1, 4);
    } else if (c.layer_depths_sorted) {
      // the layer i with depth(i-1) <= az < depth(i): the one the loop below selects
      const auto it = std::upper_bound(c.layer_depths.begin(), c.layer_depths.end(), az);
      const int i = static_cast<int>(it - c.layer_depths.begin()) + 1;
      if (i >= 2 && i <= in.nmat) {
        m[0] = mat_in(in, i, 2); m[1] = mat_in(in, i, 3); m[2] = mat_in(in, i, 4);
      }
    } else {
      for (int i = 2; i <= in.nmat; ++i) {
        if (az < mat_in(in, i, 1) && az >= mat_in(in, i - 1, 1)) {
          m[0] = mat_in(in, i, 2); m[1] = mat_in(in, i, 3); m[2] = mat_in(in, i, 4);
        }
      }
    }
  }
  m[4] = m[1] * m[1] * m[2];
  m[3] = m[0] * m[0] * m[2] - 2.0 * m[4];
}

int new_element(Case &c) {
  c.nodeElemIdRelation.resize(c.nodeElemIdRelation.size() + 8, 0);
  c.elemTypeArr.push_back(1);
  c.stressCompIndexArr.push_back(0);
  c.matRows.resize(c.matRows.size() + 5, 0.0);
  return static_cast<int>(c.elemTypeArr.size());
}

int32_t &conn(Case &c, int e, int k) { return c.nodeElemIdRelation[8 * static_cast<size_t>(e - 1) + (k - 1)]; }

void grow_stress(Case &c) {
  if (static_cast<int64_t>(c.stressArr.size()) < c.stressDofCount) c.stressArr.resize(c.stressDofCount, 0.0);
}

// src/library_degeneration.f90:3-55
void wedge(Case &c, const double ctr[3], int &elemCount, int plane_ids[8]) {
  const Inputs &in = c.in;
  const double t = c.dip_tan;
  const double dist = std::fabs(ctr[1] * t + ctr[2]) / c.dip_norm;
  if (!(ctr[0] > in.fxmin && ctr[0] < in.fxmax && ctr[1] > in.fymin && ctr[1] < in.fymax &&
        ctr[2] > in.fzmin && dist < kTol))
    return;
  static const int lower[8] = {5, 1, 4, 4, 6, 2, 3, 3};
  static const int upper[8] = {4, 8, 5, 5, 3, 7, 6, 6};
  c.elemTypeArr[elemCount - 1] = 11;
  for (int k = 0; k < 8; ++k) conn(c, elemCount, k + 1) = plane_ids[lower[k] - 1];
  elemCount = new_element(c);
  c.elemTypeArr[elemCount - 1] = 12;
  for (int k = 0; k < 8; ++k) conn(c, elemCount, k + 1) = plane_ids[upper[k] - 1];
  c.stressCompIndexArr[elemCount - 1] = static_cast<int32_t>(c.stressDofCount);
  c.stressDofCount += 12;
  grow_stress(c);
  double *m = &c.matRows[5 * static_cast<size_t>(elemCount - 1)];
  m[0] = mat_in(in, 1, 1); m[1] = mat_in(in, 1, 2); m[2] = mat_in(in, 1, 3);
  m[4] = m[1] * m[1] * m[2];
  m[3] = m[0] * m[0] * m[2] - 2 * m[4];
}

// src/meshgen.f90:976-995
void set_plastic_stress(Case &c, double depth, int e) {
  const Inputs &in = c.in;
  const int etTag = (c.elemTypeArr[e - 1] == 2) ? 1 : 0;
  c.eleporep[e - 1] = 0.0;
  const double strVert = -(in.roumax - in.rhow * (in.gamar + 1.0)) * depth * kGrav;
  const double devStr = std::fabs(strVert) * in.devStrToStrVertRatio;
  const int64_t b = c.stressCompIndexArr[e - 1] + 15 * etTag;  // 0-based offset, entries 1..6
  c.stressArr[b + 2] = strVert;
  c.stressArr[b + 0] = strVert - devStr * std::cos(2.0 * in.str1ToFaultAngle);
  c.stressArr[b + 1] = strVert + devStr * std::cos(2.0 * in.str1ToFaultAngle);
  c.stressArr[b + 5] = devStr * std::sin(2.0 * in.str1ToFaultAngle);
}

// src/meshgen.f90:3-156
void mesh(Case &c) {
  const Inputs &in = c.in;
  int nyuni;
  grid_line(c, 1, c.xline, c.nxuni);
  grid_line(c, 2, c.yline, nyuni);
  grid_line(c, 3, c.zline, c.nzuni);
  c.nx = static_cast<int>(c.xline.size());
  c.ny = static_cast<int>(c.yline.size());
  c.nz = static_cast<int>(c.zline.size());
  const int nxyz = c.nx * c.ny * c.nz;
  {
    // split nodes are numbered after the grid's nodes: room for one per uniform fault cell
    const size_t nodes = static_cast<size_t>(nxyz) + static_cast<size_t>(c.nxuni) * c.nzuni + 16;
    c.eqNumStartIndexLoc.reserve(nodes);
    c.numOfDofPerNodeArr.reserve(nodes);
    c.meshCoor.reserve(3 * nodes);
  }
  c.eqNumStartIndexLoc.assign(nxyz, 0);
  c.numOfDofPerNodeArr.assign(nxyz, 0);
  c.meshCoor.assign(static_cast<size_t>(3) * nxyz, 0.0);
  c.fltrc.assign(static_cast<size_t>(2) * c.nxuni * c.nzuni, 0);
  c.n4yn.assign(in.nOffSt, 0);
  c.layer_depths.clear();
  if (in.nmat > 1 && in.n2mat == 4)
    for (int i = 1; i <= in.nmat; ++i) c.layer_depths.push_back(mat_in(in, i, 1));
  c.layer_depths_sorted = !c.layer_depths.empty();
  for (size_t i = 1; i < c.layer_depths.size(); ++i)
    if (!(c.layer_depths[i] > c.layer_depths[i - 1])) c.layer_depths_sorted = false;
  c.dip_tan = std::tan(in.C_degen / 180.0 * kPi);
  c.dip_norm = std::pow(1.0 + c.dip_tan * c.dip_tan, 0.5);
  c.station_level.assign(c.nz, 0);
  for (int iz = 1; iz <= c.nz; ++iz)
    for (int i = 0; i < in.nOffSt; ++i)
      if (std::fabs(c.zline[iz - 1] - in.x4nds[3 * i + 2]) < kTol) c.station_level[iz - 1] = 1;
  {
    // capacity for one hexahedron per grid cell (wedges and split nodes may still grow these);
    // reserved pages are not touched until they are filled
    const size_t cells = static_cast<size_t>(c.nx - 1) * (c.ny - 1) * (c.nz - 1);
    c.eqNumIndexArr.reserve(static_cast<size_t>(12) * nxyz);
    c.nodeElemIdRelation.reserve(8 * cells);
    c.elemTypeArr.reserve(cells);
    c.stressCompIndexArr.reserve(cells);
    c.matRows.reserve(5 * cells);
    c.eleporep.reserve(cells);
    c.stressArr.reserve(21 * cells);
  }
  // plane1/plane2: node ids of the previous / current x-plane, indexed (iy, iz), 1-based
  std::vector<int32_t> plane1(static_cast<size_t>(c.ny + 1) * (c.nz + 1), 0), plane2 = plane1;
  auto P = [&](std::vector<int32_t> &pl, int iy, int iz) -> int32_t & {
    return pl[static_cast<size_t>(iy) + static_cast<size_t>(c.ny + 1) * iz];
  };
  int nodeCount = 0, elemCount = 0;
  c.cell_plane_start.assign(c.nx + 2, 1);
  for (int ix = 1; ix <= c.nx; ++ix) {
    c.cell_plane_start[ix] = elemCount + 1;  // first element of the cells between planes ix-1, ix
    for (int iz = 1; iz <= c.nz; ++iz) {
      for (int iy = 1; iy <= c.ny; ++iy) {
        const double p[3] = {c.xline[ix - 1], c.yline[iy - 1], c.zline[iz - 1]};
        ++nodeCount;
        P(plane2, iy, iz) = nodeCount;
        coor(c, nodeCount, 1) = p[0];
        coor(c, nodeCount, 2) = p[1];
        coor(c, nodeCount, 3) = p[2];
        if (in.insertFaultType > 0) {
          insert_fault_interface(c, p);
          coor(c, nodeCount, 2) = c.ycoort;
        }
        int ndofNode = 3;  // src/meshgen.f90:562-572
        if (p[0] > c.PMLb[0] || p[0] < c.PMLb[1] || p[1] > c.PMLb[2] || p[1] < c.PMLb[3] ||
            p[2] < c.PMLb[4])
          ndofNode = 12;
        c.eqNumStartIndexLoc[nodeCount - 1] = static_cast<int32_t>(c.eqNumIndexArr.size());
        c.numOfDofPerNodeArr[nodeCount - 1] = ndofNode;
        set_equation_numbers(c, p, ndofNode);
        surface_station(c, ix, iy, iz, p, nodeCount);
        create_master_node(c, ix, iy, iz, p, nodeCount);
        if (ix >= 2 && iy >= 2 && iz >= 2) {
          // createElement, src/meshgen.f90:702-741
          elemCount = new_element(c);
          int ids[8] = {P(plane1, iy - 1, iz - 1), P(plane2, iy - 1, iz - 1), P(plane2, iy, iz - 1),
                        P(plane1, iy, iz - 1),     P(plane1, iy - 1, iz),     P(plane2, iy - 1, iz),
                        P(plane2, iy, iz),         P(plane1, iy, iz)};
          double ctr[3] = {0, 0, 0};
          for (int k = 0; k < 8; ++k) {
            conn(c, elemCount, k + 1) = ids[k];
            for (int q = 1; q <= 3; ++q) ctr[q - 1] += coor(c, ids[k], q);
          }
          for (double &v : ctr) v /= 8.0;
          c.stressCompIndexArr[elemCount - 1] = static_cast<int32_t>(c.stressDofCount);
          if (ctr[0] > c.PMLb[0] || ctr[0] < c.PMLb[1] || ctr[1] > c.PMLb[2] ||
              ctr[1] < c.PMLb[3] || ctr[2] < c.PMLb[4]) {
            c.elemTypeArr[elemCount - 1] = 2;
            c.stressDofCount += 15 + 6;
          } else {
            c.stressDofCount += 12;
          }
          grow_stress(c);
          c.eleporep.resize(c.elemTypeArr.size(), 0.0);
          set_material(c, elemCount, ctr);
          if (in.C_degen > 3.0) {
            wedge(c, ctr, elemCount, ids);
            c.eleporep.resize(c.elemTypeArr.size(), 0.0);
            for (int q = 1; q <= 2; ++q) {
              const int nid = conn(c, elemCount, q);
              const double pq[3] = {coor(c, nid, 1), coor(c, nid, 2), coor(c, nid, 3)};
              if (on_fault(c, pq) && c.elemTypeArr[elemCount - 1] == 1) c.elemTypeArr[elemCount - 1] = 13;
            }
          }
          // replaceSlaveWithMasterNode, src/meshgen.f90:743-766
          const int et = c.elemTypeArr[elemCount - 1];
          if ((et == 1 && p[0] > in.fxmin - kTol && p[0] < in.fxmax + in.dx + kTol &&
               p[2] > in.fzmin - kTol && p[1] > 0.0 && std::fabs(p[1] - in.dy) < kTol) ||
              et == 12 || et == 13) {
            for (int k = 1; k <= 8; ++k) {
              auto it = c.slave_to_master.find(conn(c, elemCount, k));
              if (it != c.slave_to_master.end()) conn(c, elemCount, k) = it->second;
            }
          }
          if (in.C_elastic == 0)
            set_plastic_stress(c, -0.5 * (c.zline[iz - 1] + c.zline[iz - 2]) + 7.3215, elemCount);
        }
      }
    }
    plane1 = plane2;
  }
  // fault areas, src/meshgen.f90:113-152
  c.arn.assign(c.nftnd, 0.0);
  if (c.nftnd > 0) {
    auto F = [&](int j, int i, int which) -> int32_t {
      return c.fltrc[2 * (static_cast<size_t>(j - 1) + static_cast<size_t>(c.nxuni) * (i - 1)) + which];
    };
    auto dist = [&](int a, int b) {
      double s = 0;
      for (int q = 1; q <= 3; ++q) {
        const double d = coor(c, b, q) - coor(c, a, q);
        s += d * d;
      }
      return std::sqrt(s);
    };
    for (int i = 2; i <= c.ifd; ++i) {
      for (int j = 2; j <= c.ifs; ++j) {
        const int n1 = F(j, i, 0), n2 = F(j - 1, i, 0), n3 = F(j - 1, i - 1, 0), n4 = F(j, i - 1, 0);
        const int m1 = F(j, i, 1), m2 = F(j - 1, i, 1), m3 = F(j - 1, i - 1, 1), m4 = F(j, i - 1, 1);
        if (!n1 || !n2 || !n3 || !n4) fail("incomplete fault grid while computing areas");
        const double aa = dist(n1, n2), bb = dist(n2, n3), cc = dist(n3, n4), dd = dist(n4, n1);
        const double p1 = dist(n2, n4), q1 = dist(n1, n3);
        const double t = bb * bb + dd * dd - aa * aa - cc * cc;
        double area = 0.25 * std::sqrt(4 * p1 * p1 * q1 * q1 - t * t);
        area = 0.25 * area;
        c.arn[m1 - 1] += area;
        c.arn[m2 - 1] += area;
        c.arn[m3 - 1] += area;
        c.arn[m4 - 1] += area;
      }
    }
  }
  // consistency checks, src/meshgen.f90:405-435 and src/eqdyna3d.f90:214-224
  const int nelem = static_cast<int>(c.elemTypeArr.size());
  for (int e = 0; e < nelem; ++e) {
    const double *m = &c.matRows[5 * static_cast<size_t>(e)];
    if (m[0] == 0.0 || m[1] == 0.0 || m[2] == 0.0) fail("element without material property");
  }
  c.cell_plane_start[c.nx + 1] = nelem + 1;
  c.pstrain.assign(nelem, 0.0);
  c.eleporep.resize(nelem, 0.0);
  c.stressArr.resize(std::max<int64_t>(c.stressDofCount, 1), 0.0);
}

// src/netcdf_io.f90:70-106
void on_fault_fields(Case &c) {
  const Inputs &in = c.in;
  const int fnx = static_cast<int>(fnint((in.fxmax - in.fxmin) / in.dx)) + 1;
  const int fnz = static_cast<int>(fnint((in.fzmax - in.fzmin) / in.dz)) + 1;
  if (fnx != in.ofv_nfx || fnz != in.ofv_nfz)
    fail("on_fault_vars_input.bin has " + std::to_string(in.ofv_nfx) + "x" +
         std::to_string(in.ofv_nfz) + " points, the fault grid needs " + std::to_string(fnx) +
         "x" + std::to_string(fnz));
  const int n = c.nftnd;
  c.fric.assign(static_cast<size_t>(100) * std::max(n, 1), 0.0);
  c.fnft.assign(std::max(n, 1), 99999.0);
  auto V = [&](int ii, int jj, int var) {  // on_fault_vars(ii, jj, var), 1-based
    return in.ofv[static_cast<size_t>(ii - 1) + static_cast<size_t>(fnx) * ((jj - 1) + static_cast<size_t>(fnz) * (var - 1))];
  };
  for (int i = 1; i <= n; ++i) {
    const int s = c.nsmp[2 * (i - 1)];
    const double xc = coor(c, s, 1), zc = coor(c, s, 3);
    const int ii = static_cast<int>(fnint((xc - in.fxmin) / in.dx)) + 1;
    const int jj = static_cast<int>(fnint((zc - in.fzmin) / in.dz)) + 1;
    if (ii < 1 || ii > fnx || jj < 1 || jj > fnz) fail("fault node outside on_fault_vars grid");
    double *f = &c.fric[100 * static_cast<size_t>(i - 1) - 1];  // f[k] == fric(k,i)
    f[1] = V(ii, jj, 1);   f[2] = V(ii, jj, 2);   f[3] = V(ii, jj, 3);
    f[9] = V(ii, jj, 4);   f[10] = V(ii, jj, 5);  f[11] = V(ii, jj, 6);
    f[12] = V(ii, jj, 7);  f[13] = V(ii, jj, 8);  f[14] = V(ii, jj, 9);
    f[15] = V(ii, jj, 10); f[16] = V(ii, jj, 11); f[17] = V(ii, jj, 12);
    f[18] = V(ii, jj, 13); f[19] = V(ii, jj, 14); f[40] = V(ii, jj, 15);
    f[41] = V(ii, jj, 16); f[42] = V(ii, jj, 17); f[46] = V(ii, jj, 18);
    f[8] = V(ii, jj, 19);  f[7] = V(ii, jj, 20);  f[20] = V(ii, jj, 21);
    f[47] = f[46];
    f[25] = 0.0;
    f[26] = f[46];
    f[27] = 0.0;
    f[5] = V(ii, jj, 22);  f[4] = V(ii, jj, 23);  f[49] = V(ii, jj, 24);
    const double tau = std::hypot(f[8], f[49]);
    if (in.vini_along_shear && tau > 0.0) {
      f[26] = f[46] * f[8] / tau;
      f[27] = f[46] * f[49] / tau;
    }
    f[23] = std::fabs(f[7]);
  }
}

// src/assembleGlobalMass.f90:12-38 with the routines it calls; the per-element math is
// eqd::geom::element_tables (eqd_geometry.h), shared with the device table build.
void element_tables(Case &c) {
  const int nelem = static_cast<int>(c.elemTypeArr.size());
  const int nnode = static_cast<int>(c.eqNumStartIndexLoc.size());
  // every entry is written by the element loop below
  c.eledet.resize(nelem);
  c.elemass.resize(static_cast<size_t>(24) * nelem);
  c.eleshp.resize(static_cast<size_t>(24) * nelem);
  c.ss.resize(static_cast<size_t>(6) * nelem);
  c.phi.resize(static_cast<size_t>(32) * nelem);
  c.nodalMassArr.assign(std::max(c.equationNumCount, 1), 0.0);
  c.fnms.assign(nnode, 0.0);
  // Per-element tables are independent: computed in parallel.  The first element with a
  // non-positive determinant is reported after the loop (an exception cannot leave it).
  int bad = nelem + 1;
#pragma omp parallel for schedule(static) reduction(min : bad)
  for (int e = 1; e <= nelem; ++e) {
    double xl[3][8];
    for (int k = 0; k < 8; ++k)
      for (int q = 0; q < 3; ++q) xl[q][k] = coor(c, conn(c, e, k + 1), q + 1);
    const size_t eo = static_cast<size_t>(e - 1);
    double em[8], det = 0.0;
    if (!eqd::geom::element_tables(xl, c.elemTypeArr[e - 1], &c.matRows[5 * eo], &c.eleshp[24 * eo], det, em,
                                   &c.ss[6 * eo], &c.phi[32 * eo])) {
      bad = std::min(bad, e);
      continue;
    }
    c.eledet[e - 1] = det;
    for (int k = 0; k < 8; ++k)
      for (int q = 0; q < 3; ++q) c.elemass[24 * eo + 3 * k + q] = em[k];
  }
  if (bad <= nelem) fail("non-positive determinant at element " + std::to_string(bad));
  // nodal mass, src/assembleGlobalMass.f90:283-326.  The reference adds the element masses
  // element by element; every sum here is taken in that order.  Nodes are numbered x-plane by
  // x-plane (a split node lies in the plane of its grid node) and the elements of a layer of cells
  // touch only its two bounding planes, so the nodes of plane j receive contributions only from
  // layers j and j + 1: each plane is assembled on its own, in element order.
  const int plane_nodes = c.ny * c.nz, nxyz = c.nx * c.ny * c.nz;
  std::vector<int32_t> split_plane(c.nftnd);
  for (int k = 0; k < c.nftnd; ++k) split_plane[k] = (c.nsmp[2 * k] - 1) / plane_nodes + 1;
  auto plane_of = [&](int nid) {
    return nid <= nxyz ? (nid - 1) / plane_nodes + 1 : split_plane[nid - nxyz - 1];
  };
  int fixed_dof = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : fixed_dof)
  for (int j = 1; j <= c.nx; ++j) {
    const int e_end = c.cell_plane_start[std::min(j + 1, c.nx) + 1];
    for (int e = c.cell_plane_start[j]; e < e_end; ++e) {
      const double *em = &c.elemass[24 * static_cast<size_t>(e - 1)];
      for (int k = 0; k < 8; ++k) {
        const int nid = conn(c, e, k + 1);
        if (plane_of(nid) != j) continue;
        const int loc = c.eqNumStartIndexLoc[nid - 1];
        if (c.numOfDofPerNodeArr[nid - 1] == 12) {
          for (int q = 0; q < 3; ++q) {
            for (int d = 3 * q; d < 3 * q + 3; ++d) {
              const int eq = c.eqNumIndexArr[loc + d];
              if (eq > 0) c.nodalMassArr[eq - 1] += em[3 * k + q];
            }
            const int eq = c.eqNumIndexArr[loc + q + 9];
            if (eq > 0) c.nodalMassArr[eq - 1] += em[3 * k + q];
          }
        } else {
          for (int q = 0; q < 3; ++q) {
            const int eq = c.eqNumIndexArr[loc + q];
            if (eq > 0) c.nodalMassArr[eq - 1] += em[3 * k + q];
            else fixed_dof = 1;
          }
        }
        c.fnms[nid - 1] += em[3 * k];
      }
    }
  }
  if (fixed_dof) fail("3-DOF node with a fixed DOF is not supported");
  // wedge sanity check, src/assembleGlobalMass.f90:43-55
  for (int e = 1; e <= nelem; ++e) {
    const int et = c.elemTypeArr[e - 1];
    if (et >= 11 && et <= 12 && conn(c, e, 3) != conn(c, e, 4)) fail("wrongly created wedge");
  }
}

// The checks of element_tables that do not need the tables (a mesh-only build): wedge sanity,
// src/assembleGlobalMass.f90:43-55.
void mesh_checks(Case &c) {
  const int nelem = static_cast<int>(c.elemTypeArr.size());
  for (int e = 1; e <= nelem; ++e) {
    const int et = c.elemTypeArr[e - 1];
    if (et >= 11 && et <= 12 && conn(c, e, 3) != conn(c, e, 4)) fail("wrongly created wedge");
  }
}

void finish(Case &c) {
  const Inputs &in = c.in;
  const int nnode = static_cast<int>(c.eqNumStartIndexLoc.size());
  const int nelem = static_cast<int>(c.elemTypeArr.size());
  const int neq = std::max(c.equationNumCount, 1);
  // mat (nelem, 5), column-major
  c.mat.resize(static_cast<size_t>(5) * nelem);
#pragma omp parallel for schedule(static)
  for (int e = 0; e < nelem; ++e)
    for (int k = 0; k < 5; ++k) c.mat[static_cast<size_t>(k) * nelem + e] = c.matRows[5 * static_cast<size_t>(e) + k];
  std::vector<double>().swap(c.matRows);  // the case lives as long as its arrays: drop the copy
  c.n_phys_elem = 0;
  for (int e = 0; e < nelem; ++e) c.n_phys_elem += (c.elemTypeArr[e] != 2);
  zero_fill(c.v1, neq);
  zero_fill(c.nodalForceArr, neq);
  zero_fill(c.velArr, static_cast<size_t>(3) * nnode);
  zero_fill(c.dispArr, static_cast<size_t>(3) * nnode);
  // init_vel, src/eqdyna3d.f90:191-212
  for (int i = 1; i <= c.nftnd; ++i) {
    const double *f = &c.fric[100 * static_cast<size_t>(i - 1) - 1];
    const int ls = c.eqNumStartIndexLoc[c.nsmp[2 * (i - 1)] - 1];
    const int lm = c.eqNumStartIndexLoc[c.nsmp[2 * (i - 1) + 1] - 1];
    for (int q = 0; q < 3; ++q) {
      c.v1[c.eqNumIndexArr[ls + q] - 1] = f[34 + q];
      c.v1[c.eqNumIndexArr[lm + q] - 1] = f[31 + q];
    }
  }
  // derived scalars, src/readInputFiles.f90:182-186
  const int nstep = static_cast<int>(fnint(in.totalSimuTime / in.dt));
  // station index rows, src/eqdyna3d.f90:169-188
  c.idhist.clear();
  for (int s = 0; s < c.numOffFaultSt; ++s)
    for (int d = 1; d <= 3; ++d)
      for (int dv = 1; dv <= 2; ++dv) {
        c.idhist.push_back(c.offStIndex[2 * s + 1]);
        c.idhist.push_back(d);
        c.idhist.push_back(dv);
      }
  c.onFaultQuantHistSCECForm.assign(static_cast<size_t>(12) * nstep * std::max(c.numOnFaultSt, 1), 0.0);
  if (c.numOffFaultSt > 0)
    c.OffFaultStGramSCEC.assign(static_cast<size_t>(6 * c.numOffFaultSt + 1) * nstep, 0.0);
  const size_t tp = static_cast<size_t>(2) * std::max(c.nftnd, 1) * nstep;
  if (in.friclaw == 5 || (in.friclaw >= 3 && tp <= (static_cast<size_t>(1) << 26)))
    c.onFaultTPHist.assign(tp, 0.0);

  eqd_scalars &s = c.sc;
  std::memset(&s, 0, sizeof(s));
  s.dt = in.dt;
  s.rdampk = in.rdampk * in.dt;
  s.rdampm = in.rdampm;
  s.grav = kGrav;
  s.roumax = in.roumax;
  s.rhow = in.rhow;
  s.gamar = in.gamar;
  s.w = 8.0;
  s.kapa_hg = in.kapa_hg;
  s.xsource = in.xsource;
  s.ysource = in.ysource;
  s.zsource = in.zsource;
  s.nucR = in.nucR;
  s.nucRuptVel = in.nucRuptVel;
  s.nucdtau0 = in.nucdtau0;
  s.nucT = in.nucT;
  for (int k = 0; k < 8; ++k) s.PMLb[k] = c.PMLb[k];
  s.vmaxPML = in.vmaxPML;
  s.R = in.R;
  s.ccosphi = in.coheplas * std::cos(std::atan(in.bulk));
  s.sinphi = std::sin(std::atan(in.bulk));
  s.tv = 2.0 * in.dz / 3464.0;
  s.dx = in.dx;
  s.slipRateThres = in.slipRateThres;
  s.fric_tp_h = 0.0;  // never assigned in the reference (src/globalvar.f90:42)
  s.time0 = 0.0;
  s.C_elastic = in.C_elastic;
  s.C_Q = in.C_Q;
  s.C_hg = in.C_hg;
  s.friclaw = in.friclaw;
  s.TPV = in.TPV;
  s.C_nuclea = in.C_nuclea;
  s.nucfault = in.nucfault;
  s.insertFaultType = in.insertFaultType;
  s.nPML = in.nPML;
  s.nstep = nstep;
  s.mode = in.mode;
}

}  // namespace

struct eqd_case {
  Case c;
  double phase_s[5] = {0, 0, 0, 0, 0};  // inputs, mesh, on-fault fields, element tables, finish
};

extern "C" {

const char *eqd_case_last_error(void) { return g_case_error.c_str(); }

int eqd_case_build(const char *dir, eqd_case **out) { return eqd_case_build_opt(dir, 0, out); }

int eqd_case_build_opt(const char *dir, int32_t flags, eqd_case **out) {
  if (!dir || !out) return EQD_ERR_INPUT;
  *out = nullptr;
  auto *h = new eqd_case();
  try {
    auto t = std::chrono::steady_clock::now();
    auto lap = [&](int k) {
      const auto now = std::chrono::steady_clock::now();
      h->phase_s[k] = std::chrono::duration<double>(now - t).count();
      t = now;
    };
    read_inputs(dir, h->c.in);
    lap(0);
    mesh(h->c);
    lap(1);
    on_fault_fields(h->c);
    lap(2);
    if (flags & EQD_CASE_MESH_ONLY) mesh_checks(h->c);
    else element_tables(h->c);
    lap(3);
    finish(h->c);
    lap(4);
  } catch (const CaseError &e) {
    g_case_error = e.what();
    delete h;
    return e.code;
  } catch (const std::exception &e) {
    g_case_error = e.what();
    delete h;
    return EQD_ERR_INPUT;
  }
  *out = h;
  return EQD_OK;
}

int eqd_case_view(eqd_case *h, eqd_scalars *s, eqd_host_arrays *a) {
  if (!h) return EQD_ERR_INPUT;
  Case &c = h->c;
  if (s) *s = c.sc;
  if (!a) return EQD_OK;
  std::memset(a, 0, sizeof(*a));
  a->nnode = static_cast<int32_t>(c.eqNumStartIndexLoc.size());
  a->nelem = static_cast<int32_t>(c.elemTypeArr.size());
  a->neq = c.equationNumCount;
  a->size_eqidx = static_cast<int32_t>(c.eqNumIndexArr.size());
  a->size_stress = static_cast<int64_t>(c.stressArr.size());
  a->nodeElemIdRelation = c.nodeElemIdRelation.data();
  a->elemTypeArr = c.elemTypeArr.data();
  a->eqNumIndexArr = c.eqNumIndexArr.data();
  a->eqNumStartIndexLoc = c.eqNumStartIndexLoc.data();
  a->numOfDofPerNodeArr = c.numOfDofPerNodeArr.data();
  a->meshCoor = c.meshCoor.data();
  a->eleshp = c.eleshp.empty() ? nullptr : c.eleshp.data();
  a->eledet = c.eledet.empty() ? nullptr : c.eledet.data();
  a->mat = c.mat.data();
  a->elemass = c.elemass.empty() ? nullptr : c.elemass.data();
  a->ss = c.ss.empty() ? nullptr : c.ss.data();
  a->phi = c.phi.empty() ? nullptr : c.phi.data();
  a->stressArr = c.stressArr.data();
  a->stressCompIndexArr = c.stressCompIndexArr.data();
  a->pstrain = c.pstrain.data();
  a->eleporep = c.eleporep.data();
  a->nodalMassArr = c.nodalMassArr.empty() ? nullptr : c.nodalMassArr.data();
  a->fnms = c.fnms.empty() ? nullptr : c.fnms.data();
  a->v1 = c.v1.data();
  a->velArr = c.velArr.data();
  a->dispArr = c.dispArr.data();
  a->nodalForceArr = c.nodalForceArr.data();
  a->ntotft = 1;
  a->nftmx = std::max(c.nftnd, 1);
  a->nftnd = &c.nftnd;
  a->nsmp = c.nsmp.empty() ? nullptr : c.nsmp.data();
  a->un = c.un.empty() ? nullptr : c.un.data();
  a->us = c.us.empty() ? nullptr : c.us.data();
  a->ud = c.ud.empty() ? nullptr : c.ud.data();
  a->arn = c.arn.empty() ? nullptr : c.arn.data();
  a->fric = c.fric.data();
  a->fnft = c.fnft.data();
  a->numOnFaultSt = c.numOnFaultSt;
  a->numOffFaultSt = c.numOffFaultSt;
  a->anonfs = c.anonfs.empty() ? nullptr : c.anonfs.data();
  a->idhist = c.idhist.empty() ? nullptr : c.idhist.data();
  a->onFaultQuantHistSCECForm = c.onFaultQuantHistSCECForm.data();
  a->OffFaultStGramSCEC = c.OffFaultStGramSCEC.empty() ? nullptr : c.OffFaultStGramSCEC.data();
  a->onFaultTPHist = c.onFaultTPHist.empty() ? nullptr : c.onFaultTPHist.data();
  return EQD_OK;
}

int64_t eqd_case_array_len(eqd_case *h, const char *name, int32_t *elem_bytes) {
  if (!h || !name) return 0;
  Case &c = h->c;
  struct Entry {
    const char *n;
    int64_t len;
    int32_t bytes;
  };
  const Entry table[] = {
      {"nodeElemIdRelation", (int64_t)c.nodeElemIdRelation.size(), 4},
      {"elemTypeArr", (int64_t)c.elemTypeArr.size(), 4},
      {"eqNumIndexArr", (int64_t)c.eqNumIndexArr.size(), 4},
      {"eqNumStartIndexLoc", (int64_t)c.eqNumStartIndexLoc.size(), 4},
      {"numOfDofPerNodeArr", (int64_t)c.numOfDofPerNodeArr.size(), 4},
      {"meshCoor", (int64_t)c.meshCoor.size(), 8},
      {"eleshp", (int64_t)c.eleshp.size(), 8},
      {"eledet", (int64_t)c.eledet.size(), 8},
      {"mat", (int64_t)c.mat.size(), 8},
      {"elemass", (int64_t)c.elemass.size(), 8},
      {"ss", (int64_t)c.ss.size(), 8},
      {"phi", (int64_t)c.phi.size(), 8},
      {"stressArr", (int64_t)c.stressArr.size(), 8},
      {"stressCompIndexArr", (int64_t)c.stressCompIndexArr.size(), 4},
      {"pstrain", (int64_t)c.pstrain.size(), 8},
      {"eleporep", (int64_t)c.eleporep.size(), 8},
      {"nodalMassArr", (int64_t)c.nodalMassArr.size(), 8},
      {"fnms", (int64_t)c.fnms.size(), 8},
      {"v1", (int64_t)c.v1.size(), 8},
      {"velArr", (int64_t)c.velArr.size(), 8},
      {"dispArr", (int64_t)c.dispArr.size(), 8},
      {"nodalForceArr", (int64_t)c.nodalForceArr.size(), 8},
      {"nftnd", 1, 4},
      {"nsmp", (int64_t)c.nsmp.size(), 4},
      {"un", (int64_t)c.un.size(), 8},
      {"us", (int64_t)c.us.size(), 8},
      {"ud", (int64_t)c.ud.size(), 8},
      {"arn", (int64_t)c.arn.size(), 8},
      {"fric", (int64_t)c.fric.size(), 8},
      {"fnft", (int64_t)c.fnft.size(), 8},
      {"anonfs", (int64_t)c.anonfs.size(), 4},
      {"idhist", (int64_t)c.idhist.size(), 4},
      {"onFaultQuantHistSCECForm", (int64_t)c.onFaultQuantHistSCECForm.size(), 8},
      {"OffFaultStGramSCEC", (int64_t)c.OffFaultStGramSCEC.size(), 8},
      {"onFaultTPHist", (int64_t)c.onFaultTPHist.size(), 8},
  };
  for (const Entry &e : table) {
    if (std::strcmp(e.n, name) == 0) {
      if (elem_bytes) *elem_bytes = e.bytes;
      return e.len;
    }
  }
  if (elem_bytes) *elem_bytes = 0;
  return 0;
}

int eqd_case_dims(eqd_case *h, int32_t *nx, int32_t *ny, int32_t *nz, int64_t *n_phys_elem,
                  int32_t *nstep) {
  if (!h) return EQD_ERR_INPUT;
  if (nx) *nx = h->c.nx;
  if (ny) *ny = h->c.ny;
  if (nz) *nz = h->c.nz;
  if (n_phys_elem) *n_phys_elem = h->c.n_phys_elem;
  if (nstep) *nstep = h->c.sc.nstep;
  return EQD_OK;
}

int eqd_case_lines(eqd_case *h, const double **x, const double **y, const double **z) {
  if (!h) return EQD_ERR_INPUT;
  if (x) *x = h->c.xline.data();
  if (y) *y = h->c.yline.data();
  if (z) *z = h->c.zline.data();
  return EQD_OK;
}

int eqd_case_phase_seconds(eqd_case *h, double out[5]) {
  if (!h || !out) return EQD_ERR_INPUT;
  for (int k = 0; k < 5; ++k) out[k] = h->phase_s[k];
  return EQD_OK;
}

void eqd_case_free(eqd_case *h) { delete h; }

}  // extern "C"
