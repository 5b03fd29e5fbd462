/*
 * eqdyna_gb300 — C ABI of the GB300 explicit-dynamics hot path of EQdyna.
 *
 * The reference time loop is the argument-less Fortran subroutine `driver`
 * (src/driver.f90:9-34), which mutates module `globalvar` (src/globalvar.f90:81-101).
 * This ABI replaces lines src/driver.f90:19-29 (velDispUpdate -> storeOffFaultStData ->
 * zero force -> assembleGlobalKU -> hrglss -> [thermop] -> faulting -> divide by mass).
 *
 * Conventions (identical to the Fortran arrays, so a bind(C) interface can pass them as is):
 *   - every array is column-major with the Fortran shape given in the comment;
 *   - index VALUES are 1-based (node ids, equation numbers); -1 in eqNumIndexArr is a fixed DOF
 *     (src/meshgen.f90:667-671); eqNumStartIndexLoc and stressCompIndexArr are 0-based offsets
 *     exactly as the Fortran stores them;
 *   - all reals are IEEE binary64, all integers int32 (Fortran integer(kind=4)).
 * Every entry point returns 0 on success or a positive eqd_status code; none of them exits the
 * process.  Calls are blocking, not re-entrant on one context, one device per process.
 */
#ifndef EQDYNA_GB300_H
#define EQDYNA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
enum eqd_status {
  EQD_OK = 0,
  EQD_ERR_INPUT = 1,        /* inconsistent sizes, bad pointer, unsupported option          */
  EQD_ERR_CUDA = 2,         /* a CUDA runtime call failed                                   */
  EQD_ERR_OOM = 3,          /* device allocation failed                                     */
  EQD_ERR_NAN = 4,          /* NaN velocity (src/driver.f90:147-152 stops the run)          */
  EQD_ERR_UNSUPPORTED = 5,  /* option combination not built                                  */
  EQD_ERR_NO_DEVICE = 6,    /* no CUDA device visible                                       */
  EQD_ERR_TIMEOUT = 7,      /* a bounded device wait gave up                                */
  EQD_ERR_STATE = 8         /* call out of order (step before init, ...)                    */
};

/* ---- scalar switches and constants read by the hot path ----------------------------------- */
typedef struct eqd_scalars {
  double dt;              /* time step (src/readInputFiles.f90:45)                              */
  double rdampk;          /* stiffness-proportional damping, ALREADY multiplied by dt
                             (src/readInputFiles.f90:185)                                       */
  double rdampm;          /* mass-proportional damping (src/globalvar.f90:16, 0 by default)      */
  double grav, roumax, rhow, gamar; /* gravity body force of the plastic form
                             (src/assembleGlobalKU.f90:16)                                       */
  double w;               /* one-point Gauss weight, 8 (src/calcLocalShapeFunc.f90:19)           */
  double kapa_hg;         /* viscous hourglass coefficient (src/globalvar.f90:30)               */
  double xsource, ysource, zsource, nucR, nucRuptVel, nucdtau0, nucT; /* nucleation           */
  double PMLb[8];         /* PML bounds and edge cell sizes (src/meshgen.f90:532-548)           */
  double vmaxPML, R;      /* PML reference speed and reflection coefficient                    */
  double ccosphi, sinphi, tv; /* Drucker-Prager constants (src/readInputFiles.f90:182-186)     */
  double dx;              /* uniform cell size, used by the Q mechanism index                   */
  double slipRateThres;   /* rupture-time threshold (src/faulting.f90:336)                      */
  double fric_tp_h;       /* global TP width used by thermop (src/thermop.f90:23-31)            */
  double time0;           /* timeElapsed before the first step                                   */
  /* C_Q: 0 elastic, 1 the reference's coarse-grained Q (Qs 10 above 1 km depth, 50 below; Qp = 2 Qs;
   * not with plasticity, src/warning.f90:6-9), 2 an extension with no reference counterpart:
   * Qs = 50 Vs (km/s), Qp = 2 Qs, also with plasticity. */
  int32_t C_elastic, C_Q, C_hg, friclaw, TPV, C_nuclea, nucfault, insertFaultType;
  int32_t nPML, nstep, mode, reserved;
} eqd_scalars;

/* ---- the Fortran globalvar arrays touched by the time loop --------------------------------- */
typedef struct eqd_host_arrays {
  int32_t nnode;          /* totalNumOfNodes                                                     */
  int32_t nelem;          /* totalNumOfElements                                                  */
  int32_t neq;            /* totalNumOfEquations                                                 */
  int32_t size_eqidx;     /* sizeOfEqNumIndexArr                                                 */
  int64_t size_stress;    /* size of stressArr                                                   */
  const int32_t *nodeElemIdRelation; /* (8, nelem)                                               */
  const int32_t *elemTypeArr;        /* (nelem): 1 hex, 2 PML, 11/12 wedge, 13 hex on dip fault  */
  const int32_t *eqNumIndexArr;      /* (size_eqidx)                                              */
  const int32_t *eqNumStartIndexLoc; /* (nnode)                                                   */
  const int32_t *numOfDofPerNodeArr; /* (nnode): 3 or 12                                          */
  const double *meshCoor;            /* (3, nnode)                                                */
  const double *eleshp;              /* (3, 8, nelem) global shape-function gradients             */
  const double *eledet;              /* (nelem)                                                   */
  const double *mat;                 /* (nelem, 5): vp, vs, rho, lambda, mu — element-major!     */
  const double *elemass;             /* (24, nelem)                                               */
  const double *ss;                  /* (6, nelem) hourglass stiffness                            */
  const double *phi;                 /* (8, 4, nelem) hourglass base vectors                      */
  double *stressArr;                 /* (size_stress): 12 per element, 21 per PML element         */
  const int32_t *stressCompIndexArr; /* (nelem)                                                   */
  double *pstrain;                   /* (nelem)                                                   */
  const double *eleporep;            /* (nelem)                                                   */
  const double *nodalMassArr;        /* (neq)                                                     */
  const double *fnms;                /* (nnode)                                                   */
  double *v1;                        /* (neq) velocity per equation                               */
  double *velArr;                    /* (3, nnode)                                                */
  double *dispArr;                   /* (3, nnode)                                                */
  double *nodalForceArr;             /* (neq) holds acceleration between steps                    */
  /* split-node fault */
  int32_t ntotft, nftmx;
  const int32_t *nftnd;              /* (ntotft)                                                  */
  const int32_t *nsmp;               /* (2, nftmx, ntotft): slave, master node ids                */
  const double *un, *us, *ud;        /* (3, nftmx, ntotft) unit vectors                           */
  const double *arn;                 /* (nftmx, ntotft) nodal fault area                          */
  double *fric;                      /* (100, nftmx, ntotft)                                      */
  double *fnft;                      /* (nftmx, ntotft) rupture time                              */
  /* stations */
  int32_t numOnFaultSt;              /* numOfOnFaultStCount                                       */
  int32_t numOffFaultSt;             /* numOfOffFaultStCount                                      */
  const int32_t *anonfs;             /* (3, numOnFaultSt)                                          */
  const int32_t *idhist;             /* (3, 6*numOffFaultSt)                                       */
  double *onFaultQuantHistSCECForm;  /* (12, nstep, max(1,numOnFaultSt))                          */
  double *OffFaultStGramSCEC;        /* (6*numOffFaultSt+1, nstep), may be NULL if no station     */
  double *onFaultTPHist;             /* (2, nftmx, nstep, ntotft), may be NULL unless friclaw>=3  */
} eqd_host_arrays;

/* ---- precision / solver options of the GPU form ------------------------------------------- */
enum eqd_precision {
  EQD_PREC_FP64 = 0,      /* plain form: every operation in binary64 (the drop-in)             */
  EQD_PREC_FP32 = 1       /* element strain/stress/hourglass in binary32 with Kahan-compensated
                             binary32 nodal sums and PML split fields; velocity/displacement
                             state, fault and Newton in binary64                               */
};

/* Element-table layout of the binary32 form (results are identical in both layouts). */
enum eqd_table_layout {
  EQD_TABLES_AUTO = 0,     /* per element group: records when it has few distinct records      */
  EQD_TABLES_STREAMED = 1, /* every element keeps its own geometry / material tables           */
  EQD_TABLES_RECORDS = 2   /* elements index a table of distinct (geometry, material) records;
                              EQD_ERR_UNSUPPORTED if a PML axis has > 65536 distinct factors    */
};

typedef struct eqd_options {
  int32_t precision;      /* enum eqd_precision                                                */
  int32_t learned_guess;  /* 1: MLP initial guess for the rate-and-state Newton (friclaw 3/4)  */
  int32_t record_tp_hist; /* 1: keep onFaultTPHist on the device (forced on for friclaw 5)     */
  int32_t tile_shape;     /* binary32 element tiles: bricks of bx | by << 8 | bz << 16 elements
                             (product 128), 0 = 4 x 8 x 4; chosen by eqdyna_gb300.autotune     */
  int32_t use_graph;      /* 1: capture the multi-step loop in a CUDA graph                    */
  int32_t device;         /* CUDA device ordinal                                               */
  int32_t table_layout;   /* enum eqd_table_layout (binary32 form only)                        */
  int32_t block_node;     /* node-update block size: 64, 128, 256 or 512; 0 = 256                */
  int32_t block_fault;    /* fault-kernel block size: 32, 64 or 128; 0 = 128                     */
  int32_t sequential_fault; /* binary32 form: 1 runs the fault phase of a step before the next
                             step's node update, in the reference's order; 0 (default) runs it
                             beside the next step's bulk node update (only the update of the split
                             nodes waits for it), with the same results                          */
} eqd_options;

typedef struct eqd_context eqd_context;

/* Replaces nothing in the reference: called once after init_vel (src/eqdyna3d.f90:70).
 * Copies every array the hot path reads into device-owned, GPU-laid-out buffers.
 * The host arrays stay owned by the caller; nothing is retained after return. */
int eqd_gpu_init(const eqd_scalars *s, const eqd_host_arrays *a, const eqd_options *opt,
                 eqd_context **ctx);

/* Replaces src/driver.f90:11 and :19-29 for steps nt_begin .. nt_begin+nsteps-1 (1-based).
 * timeElapsed is advanced by dt per step exactly as the reference accumulates it. */
int eqd_gpu_step(eqd_context *ctx, int32_t nt_begin, int32_t nsteps);

/* Copies device state back into the caller's arrays (velArr, dispArr, v1, stressArr, pstrain,
 * fric, fnft, station histories, onFaultTPHist) before the reference's output_* writers
 * (src/eqdyna3d.f90:75-79).  Pointers that are NULL in `a` are skipped. */
int eqd_gpu_fetch(eqd_context *ctx, eqd_host_arrays *a);

/* Copies only the fault state (fric, fnft) back — the cheap per-step read of a result. */
int eqd_gpu_fetch_fault(eqd_context *ctx, double *fric, double *fnft);

/* No counterpart in the reference: the per-step read of a step's result without the rest of the
 * fault state.  Copies fric(k, :) for the nrows 1-based row numbers k in rows[] into
 * dst[nrows][npair] (pair index fastest), e.g. rows 71-76 = slip, slip rate and peak slip rate.
 * dst may be pinned (eqd_host_alloc) for a direct DMA. */
int eqd_gpu_fetch_fric_rows(eqd_context *ctx, const int32_t *rows, int32_t nrows, double *dst);

/* No counterpart in the reference: a pipelined time loop, so that the device never waits for the
 * host between steps.  eqd_gpu_step_async queues the steps and returns at once (errors surface at
 * the next wait, fetch or synchronous step; not in profiling mode).  eqd_gpu_fetch_fric_rows_async
 * queues the read of the given fric rows as they stand after every step queued so far: a device
 * copy into one of two staging slots on the step stream, then the copy to dst (pinned memory from
 * eqd_host_alloc, so the copy engine overlaps the next steps) on a second stream; *ticket
 * identifies the read.  eqd_gpu_fetch_wait blocks until read `ticket` has reached dst and returns
 * the error status of the steps before it (EQD_ERR_NAN, EQD_ERR_TIMEOUT).  At most two reads are
 * outstanding: issuing a third first waits for the oldest, whose ticket can then no longer be
 * waited for (EQD_ERR_INPUT). */
int eqd_gpu_step_async(eqd_context *ctx, int32_t nt_begin, int32_t nsteps);
int eqd_gpu_fetch_fric_rows_async(eqd_context *ctx, const int32_t *rows, int32_t nrows, double *dst,
                                  int64_t *ticket);
int eqd_gpu_fetch_wait(eqd_context *ctx, int64_t ticket);

/* Output streams on the device.  The reference writes, when mod(nt, 10) == 1
 * (src/driver.f90:30-33), the velocity of every surface node (output_gm,
 * src/library_output.f90:267-279) and fric(47, :) of every pair (output_src_evol, :297-312).
 * eqd_gpu_output_setup makes every step with (nt - 1) % every == 0 write that frame into a ring of
 * ring_frames frames in device memory, inside the step (captured in the step graph); the
 * surface nodes are Fortran node numbers (1-based; surfaceNodeIdArr of find_surfaceNodeIdArr,
 * :246-262).  eqd_gpu_output_drain copies up to max_frames frames not yet drained, oldest first:
 * gm[k][n_surface][3] and src_evol[k][npair] (either may be NULL), *frames = the count,
 * *first_step = nt of the first.  Frames overwritten before a drain are skipped (first_step shows
 * the gap).  Once per context; not in ensembles. */
int eqd_gpu_output_setup(eqd_context *ctx, const int32_t *surface_nodes, int32_t n_surface, int32_t every,
                         int32_t ring_frames);
int eqd_gpu_output_drain(eqd_context *ctx, double *gm, double *src_evol, int32_t max_frames, int32_t *frames,
                         int32_t *first_step);

/* Page-locked host memory for the buffers a host program exchanges with the device every step
 * (cudaHostAlloc / cudaFreeHost); NULL or EQD_ERR_CUDA on failure. */
void *eqd_host_alloc(int64_t bytes);
int eqd_host_free(void *p);

/* Frees all device memory of the context (before MPI_Finalize, src/eqdyna3d.f90:86). */
int eqd_gpu_finalize(eqd_context *ctx);

/* Human-readable text of a status code. */
const char *eqd_gpu_status_string(int status);

/* Diagnostics: Newton iterations summed over pairs and steps, Newton ivmax hits, element
 * updates performed, kernel launches issued by the last eqd_gpu_step call. */
int eqd_gpu_stats(eqd_context *ctx, int64_t *newton_iters, int64_t *newton_maxhits,
                  int64_t *elem_updates, int64_t *kernel_launches);

/* Current simulation time of the context (timeElapsed). */
double eqd_gpu_time(eqd_context *ctx);

/* Timing of subsequent eqd_gpu_step calls: with enable = 1 every step records CUDA events on
 * the library's stream around each kernel launch (the step loop is issued as plain stream
 * launches in the reference's order, no graph, no overlap, while enabled); with enable = 3 only
 * the whole call is bracketed by events (graphs and the overlapped schedule kept; kind 0 below
 * then counts steps).  enable = 0 stops and enable = 2 resets the totals. */
int eqd_gpu_profile(eqd_context *ctx, int32_t enable);

/* Milliseconds and launch count accumulated while profiling, per kind:
 * 0 whole steps, 1 node update, 2 interior elements, 3 PML elements, 4 fault + stations. */
int eqd_gpu_kernel_time(eqd_context *ctx, int32_t kind, double *ms, int64_t *launches);

/* Rate-and-state Newton counters summed over pairs and steps since init: out[0] iterations as
 * the reference counts them (src/faulting.f90:459-516, at most 20 per solve; a repeated solve
 * counts both runs), out[1] solves that reached 20, out[2] iterations executed (the loop stops
 * early, with identical results, once an iterate repeats), out[3] solves that started from the
 * learned initial guess, out[4] of those repeated from the plain guess because the run from the
 * learned guess reached 20 iterations with the iterate still moving (last Newton step above
 * 1e-12 of the slip rate). */
int eqd_gpu_newton_counts(eqd_context *ctx, int64_t out[5]);

/* ---- learned initial guess of the rate-and-state Newton solve ------------------------------
 * No counterpart in the reference.  A 6 -> 64 -> 64 -> 1 MLP (BF16 tensor cores, FP32
 * accumulation) predicts ln(V / V_trial) of the converged slip rate from (ln V_trial, ln |state|,
 * normal traction, trial shear traction, a, b); Newton then runs to the reference's own exit
 * test from that guess.  It is trained on solves the plain method logs (friclaw 3 or 4). */
#define EQD_NEWTON_RECORD 16  /* doubles per logged solve: a b L V0 f0 fw Vw state0 fric(23)
                                 normal-traction trial-shear Tc fric(4) V_trial V iterations   */
#define EQD_MLP_PARAMS 5313   /* FP32 parameters: W1[64][16] b1[64] W2[64][64] b2[64] W3[64] b3 */
#define EQD_MLP_NORM 34       /* in_shift[8] in_scale[8] out_shift out_scale in_lo[8] in_hi[8]:
                                 the guess is used only for features inside [in_lo, in_hi], the
                                 range of the training data; elsewhere the plain guess */

typedef struct eqd_mlp_train_options {
  int32_t epochs;         /* passes over the training records                                  */
  int32_t batch;          /* records per Adam step (rounded up to a multiple of 128, >= 128)  */
  float lr;               /* Adam learning rate                                                */
  float holdout;          /* fraction of the records held out for the reported holdout loss    */
  uint64_t seed;          /* initial weights and shuffles                                      */
} eqd_mlp_train_options;

/* Logs every Newton solve of the next nsteps * stride steps, one step in `stride`, into a
 * device buffer owned by the context (nsteps * npair records); nsteps = 0 drops the log. */
int eqd_gpu_newton_log(eqd_context *ctx, int32_t nsteps, int32_t stride);
/* Number of records logged so far and, when host != NULL, copies up to cap of them. */
int eqd_gpu_newton_records(eqd_context *ctx, double *host, int64_t cap, int64_t *count);
/* Trains the guess on the logged records and enables it for the following steps.
 * epoch_loss[epochs] and holdout_loss may be NULL. */
int eqd_gpu_mlp_train(eqd_context *ctx, const eqd_mlp_train_options *opt, float *epoch_loss,
                      float *holdout_loss);
/* FP32 parameters and normalisation of the current model (either may be NULL). */
int eqd_gpu_mlp_get(eqd_context *ctx, float *params, float *norm);
/* Loads a model (e.g. saved by eqd_gpu_mlp_get) and enables it. */
int eqd_gpu_mlp_set(eqd_context *ctx, const float *params, const float *norm);
/* on = 1 uses the loaded model as the Newton initial guess, on = 0 the plain one. */
int eqd_gpu_mlp_enable(eqd_context *ctx, int32_t on);
/* Re-solves every logged record from the plain (learned = 0) or learned initial guess, with the
 * loop the fault kernel runs (fast = 1: loop-invariant law terms evaluated once, early stop on a
 * repeated iterate, same values bit for bit) or the reference's loop verbatim (fast = 0), and the
 * fault kernel's repeat from the plain guess: counts = {iterations as the reference counts them,
 * solves that reached 20, iterations executed, records, repeated solves}; v_host[records] may be
 * NULL. */
int eqd_gpu_newton_replay(eqd_context *ctx, int32_t learned, int32_t fast, int64_t counts[5],
                          double *v_host);
/* The same replay, per logged record (arrays of the record count; any may be NULL): the converged
 * slip rate, the step ratio |last Newton step| / |slip rate where it was evaluated| that decides a
 * repeat from the plain guess, and flags = iterations (as the reference counts them, both runs of
 * a repeated solve) | reached-20 << 8 | repeated-from-the-plain-guess << 9 | exit << 10, exit (the
 * fast loop only) 0 exit test or cap, 1 fixed point, 2 and 3 a 2-cycle ending on the last or on
 * the previous evaluation.  With fast = 0 and fast = 1 every field but the exit must agree. */
int eqd_gpu_newton_replay_records(eqd_context *ctx, int32_t learned, int32_t fast, double *v_host,
                                  double *step_host, int32_t *flags_host);
/* Loss sum((y - t)^2) / (2 n) and its gradient for a model and a batch, computed by the training
 * kernel: x[n][6] normalised inputs, t[n] normalised targets (gradient checks). */
int eqd_mlp_gradient(int32_t device, const float *params, const float *x, const float *t, int32_t n,
                     float *loss, float *grad);

/* Self-check of the integer-pipe conversions between binary32 and binary64 that the binary32 node
 * update uses, against the hardware conversions, over n seeded operands in each direction:
 * mismatches = {binary32 -> binary64, binary64 -> binary32} (both 0 on a correct build). */
int eqd_gpu_check_conversions(int32_t device, int64_t n, uint64_t seed, int64_t mismatches[2]);

/* ---- ensembles -----------------------------------------------------------------------------
 * No counterpart in the reference (one scenario per process there).  Several contexts created by
 * eqd_gpu_init on the same device — rupture scenarios of any mesh size and time step — advance
 * together: each step is one launch per kernel over all members (node update, interior and PML
 * elements, fault), captured in CUDA graphs.  Members must use the binary32 form with
 * record-indexed element tables (table_layout AUTO resolving to records, or RECORDS) and share the
 * physics switches (elastic/plastic, hourglass form, friction law other than 5).  Members keep their
 * own state: eqd_gpu_fetch* work on each; do not step a member by itself while it is in an
 * ensemble. */
typedef struct eqd_ensemble eqd_ensemble;
int eqd_ensemble_create(eqd_context *const *members, int32_t n, eqd_ensemble **ens);
/* Advances every member by nsteps steps (each from its own current step). */
int eqd_ensemble_step(eqd_ensemble *ens, int32_t nsteps);
int eqd_ensemble_destroy(eqd_ensemble *ens);
/* How eqd_ensemble_step runs the steps: mode 0 (default) one launch per kernel per step over all
 * members, 16 steps captured in a CUDA graph; mode 1 every step of a call (after a member's first)
 * in ONE persistent cooperative launch: the node update, interior and PML element tiles and fault
 * pairs of all members, each phase split over the resident CTAs and closed by a grid barrier whose
 * waits are bounded (a wait that gives up returns EQD_ERR_TIMEOUT from the step).  Mode 1 serves
 * slip- and time-weakening members without Q (EQD_ERR_UNSUPPORTED otherwise); results agree with
 * mode 0 to the round-off of the binary32 reductions. */
int eqd_ensemble_mode(eqd_ensemble *ens, int32_t mode);
/* Device time (ms, CUDA events on the ensemble's stream) of the last eqd_ensemble_step call. */
int eqd_ensemble_time(eqd_ensemble *ens, double *ms);

/* Wall time (ms) of the phases of eqd_gpu_init: 0 nodes (and the device context), 1 element
 * grouping and ordering, 2 element tables, 3 binary32 tiles, 4 binary32 tables and element uploads,
 * 5 fault and stations, 6-7 unused. */
int eqd_gpu_init_times(eqd_context *ctx, double ms[8]);

/* Element-table layout of the binary32 form for group 0 (interior) or 1 (PML):
 * info[0] = 2 record-indexed, 1 streamed, 0 group empty or binary64 form; info[1] = elements;
 * info[2] = distinct records; info[3] = floats per record (both 0 when streamed); info[4] = tiles;
 * info[5] = element slots (tiles x 128, empty slots included); info[6] = most distinct nodes of a
 * tile; info[7] = distinct nodes summed over the tiles (the node gathers of one pass). */
int eqd_gpu_table_info(eqd_context *ctx, int32_t group, int64_t info[8]);

/* Host only (no GPU needed): the element order the binary32 form's tiles are cut from, for group
 * 0 (interior: elemTypeArr 1 and 11-13) or 1 (PML: 2) with the given tile shape (0: default).
 * out[0 .. *n_out) = 0-based element numbers, -1 for the empty slots that pad a brick to a tile
 * boundary; *live = elements / slots (0 when the input order is kept).  With out == NULL only
 * *n_out and *live are set; a cap below *n_out returns EQD_ERR_INPUT. */
int eqd_host_element_order(const eqd_host_arrays *a, int32_t group, int32_t tile_shape, int32_t *out,
                           int64_t cap, int64_t *n_out, double *live);

/* Host only (no GPU needed): the device node order eqd_gpu_init uses.  out[0 .. *n_out) = the
 * 0-based mesh node of each device node, -1 for a padding node; counts = {split (fault) nodes,
 * first device node of the PML range (the 3-DOF range padded to a multiple of 32), PML nodes with
 * equations, device nodes (a multiple of 32)}.  Device order: split nodes of the first fault, the
 * other 3-DOF nodes, padding, PML nodes with equations, fixed PML nodes, padding; mesh order within
 * each class.  With out == NULL only *n_out and counts are set; a cap below *n_out returns
 * EQD_ERR_INPUT. */
int eqd_host_node_order(const eqd_host_arrays *a, int32_t *out, int64_t cap, int64_t *n_out, int32_t counts[4]);

/* Setup on the GPU: the per-element tables and lumped nodal masses that the reference builds on
 * the host before its time loop (assembleGlobalMass, src/assembleGlobalMass.f90:12-38,283-406;
 * calcGlobalShapeFunc, src/calcGlobalShapeFunc.f90:1-75; calcSSPhi4Hrgls,
 * src/assembleGlobalMass.f90:328-374), computed on `device` from the mesh arrays of `a` (nnode,
 * nelem, nodeElemIdRelation, elemTypeArr, meshCoor, mat; for nodalMassArr also neq,
 * eqNumIndexArr, eqNumStartIndexLoc, numOfDofPerNodeArr) and written in the Fortran layout to the
 * output arrays that are not NULL: eleshp (3, 8, nelem), eledet (nelem), elemass (24, nelem),
 * ss (6, nelem), phi (8, 4, nelem), nodalMassArr (neq), fnms (nnode).  The values are bit for bit
 * those of the reference's host arithmetic (no contraction; a node's mass is summed element by
 * element in the reference's order).  EQD_ERR_INPUT for a node id out of range or a non-positive
 * determinant.  eqd_gpu_init computes the same tables on the device when the caller passes NULL
 * for all of eleshp, eledet, elemass, ss, phi, nodalMassArr and fnms. */
int eqd_gpu_element_tables(int32_t device, const eqd_host_arrays *a, double *eleshp, double *eledet,
                           double *elemass, double *ss, double *phi, double *nodalMassArr, double *fnms);

/* No counterpart in the reference: a self-test of the failure path of the library's device-side
 * waits.  which = 0 arms an mbarrier (the kind each element tile waits on for its bulk copies) for
 * bytes that no copy delivers; which = 1 runs the persistent ensemble kernel's grid barrier with
 * one of two CTAs leaving without arriving.  The bounded wait must give up (after about 0.2 s and
 * 2 s) and flag the error word: *status = EQD_ERR_TIMEOUT, *ms = the kernel's duration.  Nothing
 * faults or hangs, and the device stays usable. */
int eqd_gpu_wait_selftest(int32_t device, int32_t which, int32_t *status, double *ms);

/* Measured binary64 fused-multiply-add throughput of a device (TFLOP/s, 2 flops per FMA),
 * from a register-resident FMA chain kernel; used as the compute roofline of the FP64 form. */
int eqd_gpu_fp64_fma_peak(int32_t device, double *tflops);

/* ---- element force pass without device allocation ------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot call cudaMalloc, e.g. a
 * Fortran program whose globalvar arrays already live on the GPU under OpenACC or CUDA Fortran
 * data management, or a host program that plans all device memory at start-up and forbids
 * allocation during the run.  Every pointer in the view is a DEVICE pointer to the Fortran array
 * named (same layout and 1-based index values as eqd_host_arrays). */
typedef struct eqd_elem_device_view {
  int32_t nnode, nelem;
  const int32_t *nodeElemIdRelation;  /* (8, nelem)                                              */
  const int32_t *elemTypeArr;         /* (nelem): only types 1, 11, 12, 13 are processed         */
  const double *eleshp;               /* (3, 8, nelem)                                           */
  const double *eledet;               /* (nelem)                                                  */
  const double *mat;                  /* (nelem, 5)                                               */
  const double *ss;                   /* (6, nelem)                                               */
  const double *phi;                  /* (8, 4, nelem)                                            */
  double *stressArr;                  /* stress(1..6) at stressCompIndexArr offsets, updated      */
  const int32_t *stressCompIndexArr;  /* (nelem)                                                  */
  const double *velArr, *dispArr;     /* (3, nnode)                                               */
  double dt, rdampk, w;               /* rdampk already multiplied by dt; w = 8                   */
  int64_t size_stress;                /* length of stressArr (bounds the stress offsets)          */
  int32_t C_elastic, C_Q, C_hg;       /* the run's switches: only 1, 0, 1 are accepted            */
} eqd_elem_device_view;

/* Maximum nnode accepted by eqd_gpu_elem_forces_noalloc (size of its fixed scratch). */
#define EQD_NOALLOC_MAX_NODES 524288

/* Elastic interior-element pass of one step (calcElemKU stress update and forces plus the
 * Kosloff-Frazier hourglass forces, binary64) on the caller's device arrays: updates stressArr in
 * place and overwrites force_out, a DEVICE array (3, nnode), with the per-node sum of the element
 * and hourglass forces.  PML elements (type 2) contribute nothing.  Valid only for the elastic
 * medium without Q and with the stiffness hourglass (C_elastic = 1, C_Q = 0, C_hg = 1); other
 * switches in the view return EQD_ERR_UNSUPPORTED before any launch.
 * Allocates no device memory: the per-node accumulator is a fixed static device array of
 * EQD_NOALLOC_MAX_NODES nodes (12 MiB, held by every GPU that loads the library until exit);
 * larger meshes are rejected with EQD_ERR_INPUT.  Work is queued on `stream` (a cudaStream_t,
 * NULL = legacy default stream) and the call waits for it to finish.  The device tables are
 * checked on the device: an element with a node id outside 1 .. nnode or a stress offset outside
 * 0 .. size_stress - 6 is skipped (its stress is not updated and it adds no force) and the call
 * returns EQD_ERR_INPUT after the others have been processed.  A CUDA error already pending when
 * the call starts is left pending and reported as EQD_ERR_CUDA, with nothing launched.  The first
 * call on a device looks up the accumulator's device address with that device current; make that
 * first call before any stream capture.  All calls on a device share the accumulator (it is
 * cleared at the start of each call), so calls whose work overlaps on the GPU race; serialise
 * them on one stream. */
int eqd_gpu_elem_forces_noalloc(const eqd_elem_device_view *view, double *force_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* EQDYNA_GB300_H */
