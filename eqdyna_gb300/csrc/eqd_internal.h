// Internal definitions shared by the translation units of libeqdyna_gb300.so.
//
// Device layout (all arrays structure-of-arrays, component-major: a[c * n + i]):
//   nodes      device id = 3-DOF nodes first (original order), then 12-DOF PML nodes (original
//              order); the PML slot of node i is i - n_int, so no lookup table is needed
//              vel, disp, F  [3][nnode]  velArr, dispArr, force accumulator (DOFs 1-3, or
//                                         DOFs 10-12 on PML nodes)
//              inv_mass      [nnode]     1 / nodal mass (0 on fixed nodes)
//              F9, v9        [9][npml]   split-field force / velocity of PML DOFs 1-9
//              vh            [3][npml]   v1 of PML DOFs 10-12
//              pml_a, pml_b  [3][npml]   1/dt - d/2 and 1/(1/dt + d/2) of the node damping
//   elements   two groups, interior (types 1, 11, 12, 13) and PML (type 2), each in original
//              order; tables SoA per group: conn[8][ne], shp[24][ne], phi[32][ne], ss[6][ne],
//              detw[ne] (= eledet * w), lam, mu, stress
//   fault      one thread per split-node pair, fric[100][np] (fric(k) at row k-1)
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "eqdyna_gb300.h"

namespace eqd {

// ---- element-group tables (FP64 form keeps double, FP32 form keeps float tables) ----------
template <typename T>
struct ElemGroup {
  int ne = 0;
  int *conn = nullptr;       // [8][ne] device node ids
  T *shp = nullptr;          // [24][ne]  (3 * a + k): d N_a / d x_k
  T *phi = nullptr;          // [32][ne]  (8 * m + a)
  T *ss = nullptr;           // [6][ne]
  T *detw = nullptr;         // [ne]
  T *lam = nullptr, *mu = nullptr;  // [ne]
  T *stress = nullptr;       // interior: [6][ne] (+[6][ne] Q memory); PML: [15][ne]
  T *stress0 = nullptr;      // PML: [6][ne] constant initial stress s(16..21), or null
  T *pml_ab = nullptr;       // PML: [6][ne] a_k = 1/dt - d_k/2, b_k = 1/(1/dt + d_k/2)
  T *em = nullptr;           // [8][ne] element mass per node (body-force term), or null
  T *hgcoef = nullptr;       // viscous hourglass coefficient [ne], or null
  double *pstrain = nullptr; // [ne] plastic strain (interior, plastic form)
  T *porep = nullptr;        // [ne]
  T *qcoef = nullptr;        // Q: [5][ne]  exp(-dt/tau), miuu, Mu, wkp, wks
  int *orig = nullptr;       // [ne] original element id (0-based)
  // tiles (binary32 form): consecutive runs of `tile` elements of a spatially compact brick
  // order; each tile lists its distinct nodes and, per node, the (element, corner) incidences
  int tile = 0, ntiles = 0, max_tile_nodes = 0;
  int ne_live = 0;                  // elements (ne counts the slots, empty padding slots included)
  int64_t sum_tile_nodes = 0;       // distinct nodes summed over the tiles
  int *tile_ne = nullptr;           // [ntiles] elements of each tile: its first slots; the rest
                                    // are empty slots that align the next tile with a brick
  int ld = 0;                       // SoA stride of the binary32 tables: ntiles * tile (padded)
  int *tile_node_ptr = nullptr;     // [ntiles + 1] offsets into tile_nodes
  int *tile_nodes = nullptr;        // device node ids, sorted, per tile
  unsigned short *tile_incp = nullptr;  // per tile: M + 1 offsets into that tile's incidences
  int *tile_incp_off = nullptr;     // [ntiles + 1] offsets into tile_incp
  unsigned short *tile_inc = nullptr;   // [ntiles * tile * 8] incidences (corner * tile + e_local)
  unsigned short *tile_slot = nullptr;  // [ntiles * tile * 8] local node of (corner, e_local)
  // record-indexed binary32 tables (nrec > 0): elements with bit-identical geometry and material
  // share one record [shp 24 | phi 32, ss 6 (or hgcoef 1) | detw, lam, mu | em 8], and the
  // per-element tables above (shp ... em, pml_ab) are not allocated
  int nrec = 0, rec_len = 0;        // records, floats per record (a multiple of 4)
  float *rec = nullptr;             // [nrec][rec_len]
  unsigned *rec_id = nullptr;       // [ld] record of each element
  unsigned *ab_id = nullptr;        // PML [2][ld]: indices of (a_k, b_k) in ab_tab, 16 bits per
                                    // axis: row 0 = i_x | i_y << 16, row 1 = i_z
  float *ab_tab = nullptr;          // PML [3][ab_stride][2]
  int ab_stride = 0;                // distinct (a_k, b_k) pairs of the most varied axis
};

constexpr int kPmlAxisMax = 65536;  // distinct PML factor pairs per axis in the record layout
constexpr int kRecMax = 80;         // floats of the longest element record

// The record of a group that has exactly one (uniform grid), passed to its kernels by value.
struct RecordParam {
  float v[kRecMax];
};

struct PairStation {
  int pair;      // 0-based pair index
  int column;    // 0-based station column of onFaultQuantHistSCECForm
};

struct Context {
  // sizes
  int nnode = 0, n_int = 0, npml = 0, nelem = 0, neq = 0;
  // device node order: split (fault) nodes [0, n_split), the other 3-DOF nodes, padding up to
  // n_int; PML nodes with equations [n_int, n_int + npml_live), fixed PML nodes, padding
  int n_split = 0, npml_live = 0;
  int npair = 0, nstep = 0, nOnSt = 0, nOffRows = 0;
  int64_t size_stress = 0;
  eqd_scalars sc{};
  eqd_options opt{};
  int fp32 = 0;
  // node state
  double *vel = nullptr, *disp = nullptr, *F = nullptr, *inv_mass = nullptr;
  double *F9 = nullptr, *v9 = nullptr, *vh = nullptr, *pml_ab = nullptr;
  float *F32 = nullptr;          // FP32 form: force accumulator [3][nnode] (replaces F)
  float *F9_32 = nullptr;        // FP32 form: split-field force accumulator [9][npml] (replaces F9)
  float *v9_32 = nullptr;        // FP32 form: PML split-field velocities [9][npml] (replaces v9)
  float *pml_ab32 = nullptr;     // FP32 form: [6][npml] node damping coefficients
  float *inv_mass32 = nullptr;   // FP32 form: [nnode]; negative marks a split (fault) node
  double *Fsplit = nullptr;      // FP32 form: binary64 forces of split nodes [3][2 * npair]
  int *split_slot = nullptr;     // FP32 form: [nnode] slot of a split node in Fsplit
  float *vel32 = nullptr;        // FP32 form: [3][nnode] velocity copy
  float *dl32 = nullptr;         // FP32 form: [3][nnode] disp + rdampk * vel copy
  int *node_orig = nullptr;      // host only: device id -> original node id (0-based)
  int *node_dev = nullptr;       // host only: original -> device id
  // elements
  ElemGroup<double> gi64, gp64;
  ElemGroup<float> gi32, gp32;
  RecordParam rec0[2] = {};     // host copy of record 0 of each binary32 group (used when nrec == 1)
  int *elem_type_host = nullptr;
  // fault
  int *pair_s = nullptr, *pair_m = nullptr;  // device node ids
  double *pair_geo = nullptr;   // [13][np]: un(3), us(3), ud(3), arn, mS, mM, radius
  double *fric = nullptr;       // [100][np]
  double *fnft = nullptr;       // [np]
  double *tp_hist = nullptr;    // (2, np, nstep) like onFaultTPHist, or null
  PairStation *onst = nullptr;  // [nOnSt]
  double *onhist = nullptr;     // (12, nstep, nOnSt)
  int *off_rows = nullptr;      // [3][nOffRows]: device node, component (0-2), type (1,2,3)
  double *offhist = nullptr;    // (nOffRows + 1, nstep)
  // MLP initial guess (rate-and-state)
  void *mlp = nullptr;           // MlpDevice (device); used by the fault kernel while mlp_on
  int mlp_on = 0;
  float *mlp_p = nullptr;        // FP32 master parameters, gradients, Adam moments [kMlpParams]
  float *mlp_g = nullptr, *mlp_m = nullptr, *mlp_v = nullptr;
  float mlp_norm[34] = {};       // in_shift[8], in_scale[8], out_shift, out_scale, in_lo[8], in_hi[8]
  long long mlp_steps = 0;       // Adam steps taken
  // logged rate-and-state Newton solves (training data of the learned guess)
  double *nlog = nullptr;        // [nlog_steps][npair][16]
  int nlog_nt0 = 0, nlog_steps = 0, nlog_stride = 1;
  // step bookkeeping
  int *d_nt = nullptr;          // current step index on the device
  int *d_nt_c = nullptr;        // its copy for the fault phase of the overlapped schedule
  int pml_touches_split = 0;    // a PML element has a split node (the PML pass then waits for
                                // the split-node update, like the interior pass)
  cudaStream_t side = nullptr;  // fault phase of the overlapped schedule
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  double *d_times = nullptr;    // [nstep + 2] timeElapsed after nt steps
  int *d_err = nullptr;         // error word: 1 = NaN velocity, 2 = bounded wait gave up
  unsigned long long *d_stats = nullptr;  // [5]: Newton iterations (as counted by the reference),
                                          // ivmax hits, iterations executed, learned guesses used,
                                          // learned solves repeated from the plain guess
  int nt = 0;                   // steps completed (host mirror)
  double time = 0.0;
  int f_is_acc = 0;             // first node update consumes acceleration (from init state)
  int64_t launches_last = 0;
  int64_t elem_updates = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  int device = 0;
  int times_cap = 0;            // entries of d_times
  // profiling (CUDA events around every launch of a step)
  int profile = 0;
  int time_calls = 0;           // events around each step call only (graphs and overlap kept)
  cudaEvent_t call_ev[2] = {nullptr, nullptr};
  std::vector<cudaEvent_t> prof_events;
  double prof_ms[5] = {0, 0, 0, 0, 0};
  int64_t prof_launches[5] = {0, 0, 0, 0, 0};
  std::vector<void *> allocs;   // every device allocation of the context
  // pipelined result reads (eqd_gpu_fetch_fric_rows_async): two staging slots, each a device copy
  // of the requested fric rows and the error word, copied to the host on copy_stream
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_staged[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
  double *d_stage[2] = {nullptr, nullptr};
  size_t stage_cap[2] = {0, 0};  // doubles
  int *h_err = nullptr;          // pinned [2]
  int64_t async_issued = 0, async_waited = 0;
  // output streams (eqd_gpu_output_setup): a ring of frames written on the device
  int out_nsurf = 0, out_every = 0, out_ring = 0;
  int *out_surf = nullptr;       // device node ids of the surface nodes
  double *out_frames = nullptr;  // [out_ring][3 out_nsurf + npair]
  int *out_count = nullptr;      // frames written so far (device)
  int64_t out_drained = 0;       // frames handed to the host
};

// ---- launchers implemented in the kernel translation units --------------------------------
int launch_node_update(Context &c, cudaStream_t s, bool skip_split = false);
int launch_elements(Context &c, cudaStream_t s, int part = 2);  // 0 interior, 1 PML, 2 both
int launch_fault(Context &c, cudaStream_t s, bool overlapped = false);
int launch_output_capture(Context &c, cudaStream_t s, int part = 3, bool overlapped = false);
int launch_split_update(Context &c, cudaStream_t s);
int launch_station_capture(Context &c, cudaStream_t s);

// Ensembles: one launch per kernel over several contexts.  *_update builds the device argument
// tables on the first call (handle == null) and refreshes them afterwards (per-member state such
// as the first-step flag, the time table, the learned guess); the launches read the tables.
struct ElemConst;
int node_fault_batch_update(void **handle, Context *const *members, int n);
int launch_node_update_batched(const void *handle, cudaStream_t s);
int launch_fault_batched(const void *handle, cudaStream_t s);
void node_fault_batch_free(void *handle);
int elem_batch_update(void **handle, Context *const *members, int n, const ElemConst *k);
int launch_elements_batched(const void *handle, cudaStream_t s, int part);
void elem_batch_free(void *handle);
// The element tables of an ensemble for the persistent kernel: device argument arrays
// (ElemArgs32 of elem32r_body.cuh) and tile prefix sums of both groups, tiles and largest tile node
// count per group, and the kernel variant {body, plastic, s0, hg, q}.
int elem_batch_tables(const void *handle, const void *args[2], const int *start[2], int tiles[2], int Mmax[2],
                      int variant[5]);
// Advances every member of an ensemble by nsteps steps (none the first of its run) in one
// cooperative launch; bar: 2 device words, zero between launches; EQD_ERR_UNSUPPORTED when a member
// runs rate-and-state friction or the binary32 Q form (the batched launches cover those).
int launch_ensemble_persistent(const void *nf, const void *eb, int nsteps, unsigned *bar, int *err,
                               cudaStream_t s);
int mlp_init(Context &c);
void mlp_free(Context &c);
int newton_log_start(Context &c, int nsteps, int stride);
long long newton_log_count(const Context &c);
int newton_records(Context &c, double *host, long long cap, long long *count);
int mlp_train(Context &c, const eqd_mlp_train_options &o, float *epoch_loss, float *holdout_loss);
int mlp_get(Context &c, float *params, float *norm);
int mlp_set(Context &c, const float *params, const float *norm);
int newton_replay(Context &c, int learned, int fast, long long counts[5], double *v_host,
                  double *step_host = nullptr, int *flag_host = nullptr);

}  // namespace eqd
