/*
 * wql.h -- C ABI of the GB300 time-stepping library for WaveQLab3D inputs.
 *
 * The reference (aaimran/waveqlab3d-gh, Fortran 2008 + MPI) advances a
 * two-block domain with
 *     do n = 1, nt; call time_step_RK(D, D%dt, RK, n); end do
 * (src/main.f90:83-85, src/time_step.f90:68-150).  This library owns the
 * device state of that domain and replaces the body of time_step_RK: the
 * five RK stages of scale_rates / set_rates / exchange_fields_interface /
 * enforce_bound_iface_conditions / update_fields (src/domain.f90:586-994),
 * the stage-1 fault output (src/domain.f90:715-806) and the plastic update
 * on the last stage.  Setup reads the reference's `.in` namelist format.
 *
 * Conventions: every function returns WQL_OK (0) or a WQL_E_* code and never
 * exits the process (the reference calls `stop`/MPI_Abort instead,
 * src/mpi3dbasic.f90:287-325).  wql_last_error() gives the message of the
 * last failure on the calling thread.  Host buffers are caller-owned;
 * device memory is owned by the scenario.  Arrays use the reference's
 * column-major point order (q fastest, then r, then s), without ghost layers.
 * Calls on one scenario must not overlap; different scenarios are
 * independent.
 */
#ifndef WQL_H
#define WQL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WQL_OK 0
#define WQL_E_INPUT 1   /* malformed input or unsupported option */
#define WQL_E_OOM 2     /* device allocation failed */
#define WQL_E_CUDA 3    /* CUDA runtime error */
#define WQL_E_NAN 4     /* non-finite values detected */
#define WQL_E_SOLVER 5  /* rate-and-state solve hit its iteration cap */
#define WQL_E_STATE 6   /* call not valid in the current state */

#define WQL_FP64 0  /* reference-matching FP64 everywhere */
#define WQL_FP32C 1 /* FP32 fields with Kahan-compensated RK update, FP64 fault */

typedef struct wql_ctx wql_ctx;
typedef struct wql_scn wql_scn;

typedef struct wql_info {
  int nq[2], nr[2], ns[2]; /* block dimensions */
  double dt;               /* time step (src/domain.f90:222-235) */
  double t;                /* current time */
  int nt;                  /* floor(t_final/dt) (src/domain.f90:494) */
  int nstep;               /* steps taken */
  int precision;           /* WQL_FP64 or WQL_FP32C */
  int frames;              /* fault frames recorded so far */
  long long device_bytes;  /* device memory held by the scenario */
} wql_info;

/* Copies the last error message of this thread into buf (NUL-terminated).
 * Returns the message length. */
int wql_last_error(char* buf, size_t n);

/* Context bound to one CUDA device.  Replaces MPI start-up
 * (src/main.f90:63, src/mpi3dbasic.f90:24-120). */
int wql_ctx_create(int device, wql_ctx** out);
int wql_ctx_destroy(wql_ctx* ctx);

/* Build a scenario from a reference `.in` file: init_domain
 * (src/domain.f90:31-564) -- namelists, grids, metrics, materials, normals,
 * boundary codes, PML slabs, interface state (src/Interface_Condition.f90:
 * 2722-2850).  precision is WQL_FP64 or WQL_FP32C.  The difference operator
 * follows &problem_list fd_type (src/RHS_Interior.f90:31-125): 'traditional'
 * (SBP-6) or 'upwind' with order = 5 or 6; other operators return WQL_E_INPUT.
 * response: 'elastic', 'plastic' (plastic_model = 'scec') or 'anelastic'
 * (&anelastic_list c, weight_exp 0 or 0.6, fref; src/material.f90:11-142). */
int wql_scenario_create_from_in(wql_ctx* ctx, const char* in_path, int precision, wql_scn** out);

/* Same, from the text of a `.in` file (relative paths resolve against
 * base_dir, which may be NULL). */
int wql_scenario_create_from_text(wql_ctx* ctx, const char* in_text, const char* base_dir,
                                  int precision, wql_scn** out);
/* Seeded geometry and media supplied by the caller instead of files.  The
 * reference reads fault surfaces and topography from text files
 * (src/grid.f90:832-1160 'read_from_memomry_fractal', :1394-1450
 * 'read_topo_from_memory') and heterogeneous media from binary files
 * (src/material.f90:706-747); here the arrays are passed in directly.  Any
 * pointer may be NULL.  Layouts are column-major without ghosts. */
typedef struct wql_media {
  const double* fault_offset;   /* nr*ns: x-displacement of the fault surface (km) */
  const double* topo_offset[2]; /* per block nq*ns: y-displacement of the r = 1 surface */
  const double* lam[2];         /* per block nq*nr*ns: Lame lambda (GPa) */
  const double* mu[2];          /* per block: shear modulus (GPa) */
  const double* rho[2];         /* per block: density (g/cm^3) */
} wql_media;

int wql_scenario_create_ex(wql_ctx* ctx, const char* in_text, const char* base_dir, int precision,
                           const wql_media* media, wql_scn** out);
int wql_scenario_destroy(wql_scn* scn);

/* Advance nsteps steps = nsteps calls of time_step_RK (src/time_step.f90:68).
 * The work is queued on the scenario's stream and the call returns without
 * waiting for it; fault frames and station records are taken to host memory
 * as their device rings fill and by the calls that return them. */
int wql_step(wql_scn* scn, int nsteps);
/* One RK stage (1..5, in order) of the current step: the body of one pass
 * of the stage loop of time_step_RK (src/time_step.f90:109-147), for parity
 * and debugging; stages 1..5 give the same result as one wql_step.
 * WQL_E_STATE for a stage out of order, and for wql_step or wql_batch_add
 * while a step is in progress. */
int wql_stage(wql_scn* scn, int stage);

/* Blocks until all queued work of the scenario finished; reports device
 * faults and non-finite state (when check_nan is nonzero). */
int wql_sync(wql_scn* scn, int check_nan);

int wql_get_info(wql_scn* scn, wql_info* info);

/* Field component comp (0..8 = vx,vy,vz,sxx,syy,szz,sxy,sxz,syz,
 * src/JU_xJU_yJU_z6.f90:16304-16314) of block (0/1) to host, as double.
 * With the plastic_flow model (response = 'plastic', plastic_model other
 * than 'scec'), comp 9 and 10 read the plastic strain rate lambda and the
 * plastic strain gammap per point (P%P(:,:,:,1:2), src/plastic.f90:141,
 * src/plastic_material.f90:38-44); otherwise they return WQL_E_STATE. */
int wql_get_field(wql_scn* scn, int block, int comp, double* host_out);
int wql_set_field(wql_scn* scn, int block, int comp, const double* host_in);

/* wql_get_field without any device allocation, for callers that must not
 * allocate device memory (cudaMalloc/cudaFree synchronise the whole device,
 * so a monitoring thread reading a scenario would stall other threads'
 * streams; a memory-capped host may have no room left).  FP32 fields are
 * widened one s plane at a time through a fixed 8 MiB device array; a block
 * whose pitched plane (pq*nr, pq = nq rounded up to a multiple of 8)
 * exceeds 1048576 points returns WQL_E_INPUT.  The first call on a device
 * resolves the array's address and must not happen during stream capture.
 * The array is shared by all calls on a device: calls that overlap in time
 * race.  The calling thread's current device is the same after the call as
 * before.  No counterpart in the reference. */
int wql_get_field_noalloc(wql_scn* scn, int block, int comp, double* host_out);

/* Interface state of block copy (0/1): what 0..3 = S(1..4), 4 = W, 5 = trup;
 * nr*ns values (src/iface.f90:13-49). */
int wql_get_iface(wql_scn* scn, int copy, int what, double* host_out);

/* Manufactured-solution error of one block at the current time (needs
 * &mms_list use_mms = T).  The reference's MMS module (src/mms.f90:77-232)
 * is never called and its norm routine returns |F| rather than the error
 * (src/fields.f90:194-218); this gives, per field component c (0..8), the
 * sums over the block's grid points of (F_c - u_exact_c)^2 in err2[c] and of
 * u_exact_c^2 in ref2[c]. */
int wql_mms_norms(wql_scn* scn, int block, double* err2, double* ref2);

/* Fault output frames in the reference's file layout
 * (src/fault_output.f90:13-122, src/mpi3dio.f90:327-364): frame-major, then
 * component, then r fastest.  what: 0 Uface(9), 1 Vface(9), 2 S(4), 3 Uhat(6),
 * 4 Vhat(6), 5 Svel(3), 6 trup(1), 7 state(1).  host_out holds
 * frames*ncomp*nr*ns floats. */
int wql_frame_count(wql_scn* scn, int* frames);
int wql_get_frames(wql_scn* scn, int what, float* host_out);

/* Seismogram stations (src/seismogram.f90): with output_seismograms = T in
 * &output_list, the positions of '!---begin:station_list---' (both blocks)
 * or of station_listU / station_listV (block 1 / 2) are mapped to grid
 * points as Find_Coordinates does (src/seismogram.f90:531-650; positions
 * with no grid point within half a cell diagonal are dropped), and every
 * output step (w_stride) records t and (vx, vy, vz) there at stage 1
 * (write_seismogram, src/seismogram.f90:460-474).  wql_station_count gives
 * the stations found in a block and the records so far; wql_station_index
 * their 1-based grid indices (3 ints each); wql_get_seismograms the records
 * as records x stations x (t, vx, vy, vz) doubles. */
int wql_station_count(wql_scn* scn, int block, int* nstations, int* nrecords);
/* Writes the outputs so far in the reference's file formats under out_dir
 * (created if missing): the eight fault streams as raw float32 frames
 * <name>_interface.{Uface,Vface,S,Uhat,Vhat,Svel,trup,state}
 * (src/fault_output.f90:12-121) when w_fault = T, and one text file per
 * station, lines (4f15.10) of t, vx, vy, vz, at
 * <station_file_directory>/block<b>/<name>_<i>_<j>_<k>_block<b>.dat, or
 * <name>_<x>_<y>_<z>.dat with station_xyz_index = T
 * (src/seismogram.f90:98-114, 368-384, 460-474).  Replaces the files. */
int wql_write_outputs(wql_scn* scn, const char* out_dir);

/* The grids of both blocks of an input, computed as wql_scenario_create
 * would, written as the raw FP64 files block_grid_<id>.X/.Y/.Z (q fastest)
 * that mesh_source = 'file' reads (init_grid_from_file,
 * src/grid.f90:146-211) -- the role of the reference's preprocessor program
 * (src/preprocessor.f90).  Host only: no device is touched.  With
 * mesh_source = 'file' a scenario reads these files from base_dir, and with
 * material_source = 'file' the files btp(i)%material_path(1:3) (lambda, mu,
 * rho, raw FP64, q fastest; src/material.f90:706-747). */
int wql_write_block_grids(const char* in_text, const char* base_dir, const char* out_dir);
int wql_station_index(wql_scn* scn, int block, int* ijk);
int wql_get_seismograms(wql_scn* scn, int block, double* host_out);

/* Autotuner: times the stencil-kernel candidates (WQL_FP32C: the TMA
 * kernel with s chunks of 12..48 planes or automatic, and on Cartesian
 * blocks that fill 40-wide tiles better both tile widths, variants 5 and 6;
 * WQL_FP64: tiled and per-point) on the scenario's own blocks, reps
 * launches each, into scratch arrays (the scenario's state is not
 * changed), applies the fastest with wql_set_tuning and returns it.
 * Results are cached per block shape, mesh type and precision. */
int wql_autotune(wql_scn* scn, int reps, int* variant, int* schunk);

/* Device memory a scenario of this `.in` text would hold once created
 * (resident) and at most while it is being created (peak: resident plus the
 * FP64 set-up arrays of one block), without allocating anything.  For
 * admission control by HBM footprint. */
int wql_estimate_device_bytes(const char* in_text, const char* base_dir, int precision, long long* resident,
                              long long* peak);

/* Continuous batching of scenarios on one device.  wql_batch_step advances
 * every member by nsteps steps: per RK stage, the stencil of every eligible
 * block of every member (FP32C, default or TMA stencil variant) is one
 * kernel launch over a packed table of (block, tile, s chunk) work, and the
 * members' fault, boundary, source and correction kernels run on their own
 * streams around it.  Members may have different sizes, physics and time
 * steps; each advances exactly as wql_step would advance it alone.  Members
 * join (wql_batch_add) and leave (wql_batch_remove) between calls; a member
 * must not be stepped on its own while it is in a batch.  wql_batch_stream
 * gives the stream that every member's work of a call joins into (for
 * timing with events).  No counterpart in the reference, which runs one
 * domain per MPI job. */
typedef struct wql_batch wql_batch;
int wql_batch_create(wql_ctx* ctx, wql_batch** out);
int wql_batch_destroy(wql_batch* b);
int wql_batch_add(wql_batch* b, wql_scn* scn);
int wql_batch_remove(wql_batch* b, wql_scn* scn);
int wql_batch_step(wql_batch* b, int nsteps);
int wql_batch_stream(wql_batch* b, uintptr_t* stream);

/* Request server (continuous batching with admission by device memory).
 * A worker thread admits submitted scenarios in arrival order while the
 * head request's peak footprint (wql_estimate_device_bytes) fits within
 * hbm_budget_bytes next to the bytes held or reserved by the admitted ones
 * (the head is always admitted when nothing is admitted); a second thread
 * creates each admitted scenario while the batch steps; the worker moves
 * created scenarios into the batch, advances all running scenarios together
 * with wql_batch_step (at most round_steps steps per round, never past a
 * member's step count), and retires each scenario when it reaches its step
 * count, keeping its station seismograms.  Requests that arrive while others
 * run join the batch at the first round after their set-up.  submit copies
 * the text and media arrays and returns at once; wait blocks until the
 * request is done (status 1) or failed (status < 0: minus its WQL_E_* code)
 * or the timeout passes (status 0); result gives one block's seismograms
 * (as wql_get_seismograms, may be NULL) and the request's arrival,
 * admission (joining the batch) and completion times in seconds since the
 * server started; stats counts admitted requests still being created as
 * queued; release frees a finished request's record; destroy finishes all
 * submitted work and stops both threads.  No counterpart in the reference. */
typedef struct wql_server wql_server;
int wql_server_create(wql_ctx* ctx, long long hbm_budget_bytes, int round_steps, wql_server** out);
int wql_server_submit(wql_server* s, const char* in_text, int precision, const wql_media* media, int nsteps,
                      long long* id);
int wql_server_wait(wql_server* s, long long id, double timeout_s, int* status);
int wql_server_result(wql_server* s, long long id, int block, int* nstations, int* nrecords, double* seis,
                      double* times);
int wql_server_release(wql_server* s, long long id);
int wql_server_stats(wql_server* s, long long* completed, long long* queued, long long* active,
                     long long* bytes_in_use);
int wql_server_destroy(wql_server* s);

/* The CUDA stream the scenario's kernels run on (cudaStream_t as integer),
 * for callers that time or order work around wql_step. */
int wql_scenario_stream(wql_scn* scn, uintptr_t* stream);

/* Per-launch timing with CUDA events on the scenario stream: enable resets
 * the record; wql_kernel_times returns the summed device time and launch
 * count since then of one kernel kind: 0 the interface (fault) kernel, 1 the
 * volume stencil kernel, 2 the correction kernels (PML, boundary and fault
 * penalties, plasticity) timed together per block and stage. */
int wql_profile(wql_scn* scn, int enable);
int wql_kernel_times(wql_scn* scn, int kind, double* ms, int* launches);

/* Volume-stencil tuning: kernel_variant 0 = default (the TMA-pipelined kernel
 * in WQL_FP32C, tiled 32x8 in WQL_FP64), 1 = per-point form (every
 * neighbour read through the caches), 2 = tiled shared-memory kernel with
 * 32x8 tiles, 3 = the same at three blocks per SM (FP32), 4 = 64x8 tiles
 * (WQL_FP32C only), 5 = TMA-pipelined kernel (two-deep stage ring;
 * WQL_FP32C only; 32x12 tiles, or 40x12 on Cartesian blocks whose q extent
 * fills 40-wide tiles better), 6 = the TMA kernel on 32x12 tiles always;
 * schunk = planes per thread block along s (0 = automatic). */
int wql_set_tuning(wql_scn* scn, int kernel_variant, int schunk);

/* Number of kernel launches the last wql_step issued per time step (for
 * launch accounting); WQL_E_STATE before the first step. */
int wql_launches_per_step(wql_scn* scn, int* launches);

#ifdef __cplusplus
}
#endif

#endif /* WQL_H */
