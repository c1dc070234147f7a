/*
 * tlbm.h -- C ABI of the GB300 lattice-Boltzmann engine.
 *
 * Drop-in boundary for the timestep path of stu314159/tLBM.  The reference exposes that path as
 * the C++ class TLBM_Partition (include/TLBM_Partition.h:33-133), driven by main() in
 * src/tLBM.cpp:7-88.  Each entry point below names the reference member it replaces.
 *
 * Conventions
 *   - Every call returns a tlbm_status (0 = success); no C++ exception crosses the ABI.  After a
 *     failure, tlbm_get_last_error() describes it.  The reference throws (runtime_error,
 *     invalid_argument, const char*) or aborts; here the same conditions return a status.
 *   - A handle owns all device memory and one CUDA stream.  Use one host thread per handle.
 *   - Like the reference, inputs are the text files params.lbm, ndType.lbm and parts.lbm in the
 *     working directory, and outputs are raw *.b_dat files written in partition-major order
 *     (MPI_File_write_at semantics: files are created, never truncated).
 *   - The whole lattice lives on one GPU.  A multi-partition parts.lbm only changes the order of
 *     the output files, exactly as the reference's per-rank writes at writeOffset would.
 *   - Output files hold the precision's output type: double for TLBM_PREC_F64, float otherwise
 *     (the reference writes its compile-time `real`, float by default).
 */
#ifndef TLBM_GB300_H
#define TLBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int tlbm_status;
enum {
  TLBM_OK = 0,
  TLBM_ERR_IO = 1,               /* a file could not be opened, read or written */
  TLBM_ERR_INVALID_ARGUMENT = 2, /* bad argument, unknown lattice string, bad option */
  TLBM_ERR_FORMAT = 3,           /* malformed params.lbm / ndType.lbm / parts.lbm */
  TLBM_ERR_OUT_OF_RANGE = 4,     /* partition id >= size, node type not in {0,1,2,3,5} */
  TLBM_ERR_CUDA = 5,             /* a CUDA runtime call or kernel launch failed */
  TLBM_ERR_NUMERIC = 6,          /* non-finite mass detected by the FP64 watchdog */
  TLBM_ERR_UNSUPPORTED = 7,      /* feature not available in this build / precision */
  TLBM_ERR_TIMEOUT = 8,          /* a bounded device-side wait gave up */
  TLBM_ERR_NO_MEMORY = 9         /* host or device allocation failed */
};

/* Storage precision of the populations (the reference's compile-time `real`,
 * include/TLBM_definitions.h:11, as a run-time choice). */
typedef enum {
  TLBM_PREC_F64 = 0,  /* double populations, double arithmetic */
  TLBM_PREC_F32 = 1,  /* float populations, float arithmetic (the reference default) */
  TLBM_PREC_BF16 = 2, /* bfloat16 storage of f_i - w_i, float collision */
  TLBM_PREC_F16 = 3,  /* half storage of f_i - w_i, float collision */
  TLBM_PREC_BF16M = 4 /* bfloat16 storage of f_i - w_i (rho + e_i.(3 j)) with (rho, 3 j) of the
                         storing cell kept as FP32 beside the populations (16 B per cell), float
                         collision */
} tlbm_precision;

/* Arithmetic flavour for TLBM_PREC_F64 / TLBM_PREC_F32. */
typedef enum {
  TLBM_ARITH_REFERENCE = 0, /* the reference's operation order and type promotions, no FMA
                               contraction: bit-identical to the CPU reference */
  TLBM_ARITH_FAST = 1       /* reassociated, FMA-contracted: same physics, not bit-identical */
} tlbm_arith;

typedef enum {
  TLBM_CLOSURE_PARAMS = 0, /* BGK; Smagorinsky iff cs > 0 (src/TLBM_Partition.cpp:785-792) */
  TLBM_CLOSURE_MLP = 1     /* learned eddy-viscosity closure (weights via tlbm_set_closure_mlp) */
} tlbm_closure;

typedef struct tlbm_options {
  int struct_size; /* sizeof(tlbm_options); lets the struct grow without breaking callers */
  int precision;   /* tlbm_precision */
  int arithmetic;  /* tlbm_arith */
  int closure;     /* tlbm_closure */
  int block_x;     /* threads per block along x; 0 = tuned by the engine */
  int block_y;     /* threads per block along y; 0 = tuned by the engine */
  int device;      /* CUDA device ordinal */
  int rbgk;        /* 1: params.lbm dynamics 2 ("RBGK", include/Problem.h:19) runs the
                      regularised BGK collision (fast arithmetic only); 0: the reference's
                      behaviour, streaming without relaxation */
  int mrt;         /* 1: params.lbm dynamics 3 ("MRT", include/Problem.h:19; no case in the
                      reference, which streams without relaxation) runs the two-rate
                      moment-space collision: stress moments at omega, moments above second
                      order at mrt_ghost_rate (fast arithmetic only) */
  float mrt_ghost_rate; /* ghost-moment rate in (0, 2), a float; <= 0 selects 1.2.  The rate
                           omega gives BGK, 1 the regularised collision. */
  int f64_pipe;    /* TLBM_PREC_F64 with TLBM_ARITH_FAST: 0 (default) collides fluid nodes in
                      exact 64-bit fixed point (double-float for the Smagorinsky rate), so no
                      FP64 instruction runs on the fluid path, and for rho_lbm in [1/2, 2) holds
                      the populations on the device as that fixed point (Q1.62; exports give
                      the nearest double, and a population of magnitude 2 or more reads back as
                      NaN); 1 collides them in FP64 arithmetic on the FP64 pipe, as boundary
                      nodes always are, with IEEE double storage.  Both meet the same bar
                      against the reference arithmetic. */
  int reserved[5];
} tlbm_options;

/* The 23 values of params.lbm in file order (Problem, include/Problem.h:18-40). */
typedef struct tlbm_problem {
  char lattice[8]; /* "D3Q15" | "D3Q19" | "D3Q27" */
  int dynamics;    /* 1 = LBGK; 2 = stream without relaxation (reference behaviour) or, with
                      tlbm_options.rbgk, regularised BGK; 3 = stream without relaxation or,
                      with tlbm_options.mrt, the two-rate moment-space collision */
  int num_ts, ts_rep_freq, warmup_ts, plot_freq;
  double cs, rho_lbm, u_lbm, omega;
  int nx, ny, nz;
  int restart_flag, time_avg_flag;
  double lx_p, ly_p, lz_p, t_conv, l_conv, p_conv;
  int p_ref_idx, ss_data_flag;
} tlbm_problem;

typedef struct tlbm_handle tlbm_handle;

/* Fills *opt with defaults: TLBM_PREC_F32, TLBM_ARITH_REFERENCE, TLBM_CLOSURE_PARAMS. */
void tlbm_default_options(tlbm_options* opt);

/* Replaces TLBM_Partition(int rank, int size, MPI_Comm) (include/TLBM_Partition.h:37,
 * src/TLBM_Partition.cpp:10-14, :77-118): reads params.lbm, ndType.lbm and parts.lbm from
 * `workdir`, builds the lattice on the GPU, writes ordering.b_dat.  `rank` must be 0 (one
 * process drives the whole lattice); `size` must exceed the largest partition id, as the
 * reference requires (src/TLBM_Partition.cpp:218-224).  Options: defaults, overridden by an
 * optional `tlbm.cfg` in workdir (lines `key value`: precision f64|f32|bf16|f16,
 * arithmetic reference|fast, block_x N, block_y N, device N, rbgk 0|1, mrt 0|1,
 * mrt_ghost_rate X). */
tlbm_status tlbm_create(const char* workdir, int rank, int size, tlbm_handle** out);

/* As tlbm_create with explicit options (tlbm.cfg is not read). */
tlbm_status tlbm_create_ex(const char* workdir, int rank, int size, const tlbm_options* opt,
                           tlbm_handle** out);

/* In-memory inputs instead of files: `nd_type` and `parts` (may be NULL = one partition) hold
 * nx*ny*nz values in global order g = x + y*nx + z*nx*ny.  Outputs go to `workdir` (may be
 * NULL: no ordering.b_dat is written and tlbm_write_data fails with TLBM_ERR_IO). */
tlbm_status tlbm_create_from_arrays(const tlbm_problem* prob, const int32_t* nd_type,
                                    const int32_t* parts, const char* workdir,
                                    const tlbm_options* opt, tlbm_handle** out);

/* Replaces ~TLBM_Partition (src/TLBM_Partition.cpp:16-45). */
tlbm_status tlbm_destroy(tlbm_handle* h);

/* Replaces take_LBM_time_step(bool isEven) (src/TLBM_Partition.cpp:910-947): one fused
 * stream-collide launch.  Call with is_even = ts % 2 as main() does (src/tLBM.cpp:53). */
tlbm_status tlbm_step(tlbm_handle* h, int is_even);

/* nsteps calls of take_LBM_time_step(ts % 2) for ts = first_ts .. first_ts+nsteps-1, issued as
 * one CUDA graph launch per call (no host work between steps). */
tlbm_status tlbm_run(tlbm_handle* h, int first_ts, int nsteps);

/* As tlbm_run, timed on the handle's stream with CUDA events; *ms = device time. */
tlbm_status tlbm_time_steps(tlbm_handle* h, int first_ts, int nsteps, float* ms);

/* Waits until every step enqueued on the handle's stream has finished; returns the first
 * asynchronous error (a step launch returns before the GPU has run it). */
tlbm_status tlbm_synchronize(tlbm_handle* h);

/* Replaces write_data() (src/TLBM_Partition.cpp:608-683): writes ux{n}, uy{n}, uz{n},
 * density{n}, Fx{n}, Fy{n}, Fz{n}.b_dat for dump n = 0, 1, ... with the macroscopic values of
 * the last step and the momentum-exchange force on the post-stream populations. */
tlbm_status tlbm_write_data(tlbm_handle* h);

/* Replaces write_time_avg_data() (src/TLBM_Partition.cpp:564-606): uAvg, vAvg, wAvg, rhoAvg
 * hold sums over all steps taken (requires time_avg_flag = 1 in params.lbm). */
tlbm_status tlbm_write_time_avg_data(tlbm_handle* h);

/* Getters of TLBM_Partition (include/TLBM_Partition.h:43-50). */
int tlbm_get_num_ts(const tlbm_handle* h);
int tlbm_get_ts_rep_freq(const tlbm_handle* h);
int tlbm_get_plot_freq(const tlbm_handle* h);
int tlbm_get_warmup_ts(const tlbm_handle* h);
int tlbm_get_num_global_nodes(const tlbm_handle* h);
int tlbm_get_time_avg_flag(const tlbm_handle* h);
int tlbm_is_restart(const tlbm_handle* h);
/* Number of (node, speed) links that cross partitions of parts.lbm (get_cut_size, :685-689):
 * what the reference would send between ranks per step; nothing is sent here. */
int tlbm_get_cut_size(const tlbm_handle* h);

/* Message for the last failure on `h` (or the last failure of a create call when h is NULL). */
const char* tlbm_get_last_error(const tlbm_handle* h);
const char* tlbm_status_string(tlbm_status s);

/* ---- inspection (tools and tests; not part of the reference surface) ---------------------- */

/* Bytes per value of output files and of the copy_* buffers below (8 or 4). */
int tlbm_output_bytes(const tlbm_handle* h);
/* The options the handle runs with, after tlbm.cfg and the defaults: *out is filled up to
 * out->struct_size bytes (set it to sizeof(tlbm_options) first). */
tlbm_status tlbm_get_options(const tlbm_handle* h, tlbm_options* out);
int tlbm_num_speeds(const tlbm_handle* h);

/* Macroscopic ux, uy, uz, rho of the last step in global node order (any pointer may be NULL). */
tlbm_status tlbm_copy_macros(tlbm_handle* h, void* ux, void* uy, void* uz, void* rho);

/* Force of calc_force (src/TLBM_Partition.cpp:174-208) on the last step, global order. */
tlbm_status tlbm_copy_force(tlbm_handle* h, void* fx, void* fy, void* fz);

/* The seven write_data fields (ux, uy, uz, rho, Fx, Fy, Fz; any pointer may be NULL) of the last
 * step, as tlbm_copy_macros + tlbm_copy_force, but the call returns once the device-to-host
 * copies are queued on the handle's copy stream: the next time steps run while they proceed.
 * The host buffers (page-locked ones from tlbm_host_alloc; pageable memory makes the copies
 * synchronous) hold the values after tlbm_synchronize(h); they must not be read or freed
 * before.  A later output computation waits for these copies. */
tlbm_status tlbm_copy_outputs_async(tlbm_handle* h, void* ux, void* uy, void* uz, void* rho,
                                    void* fx, void* fy, void* fz);

/* Page-locked host memory for the tlbm_copy_* destinations (no counterpart in the reference,
 * whose write_data goes through its own buffers): copies into it run at the host link's rate
 * (~190 GB/s on GB300 against 13-25 GB/s into fresh pageable memory).  A failure leaves *out
 * NULL, with the message in tlbm_get_last_error(NULL).  tlbm_host_free(NULL) is a no-op. */
tlbm_status tlbm_host_alloc(size_t bytes, void** out);
tlbm_status tlbm_host_free(void* p);

/* Populations in the reference's layout f[node*Q + speed] (getIDx, include/TLBM_Partition.h:57):
 * which = 0: after streaming (the reference's fOut); which = 1: after collision, before
 * streaming (the reference's fIn at the end of a step). */
tlbm_status tlbm_copy_populations(tlbm_handle* h, int which, void* out);

/* Neighbour table adj[node*Q + speed] = periodic push target (create_adj_matrix,
 * src/TLBM_Partition.cpp:254-271), computed on the GPU from the same index arithmetic the
 * stream step uses. */
tlbm_status tlbm_copy_adjacency(tlbm_handle* h, int32_t* out);

/* Total mass sum_{node,speed} f as a deterministic FP64 reduction on the GPU. */
tlbm_status tlbm_mass(tlbm_handle* h, double* mass);

/* Number of kernels this handle has launched since creation. */
int64_t tlbm_kernel_launches(const tlbm_handle* h);

/* Replaces load_restart_data (src/TLBM_Partition.cpp:481-540): sets both population buffers
 * to the equilibrium of the given macroscopic fields (float, global order, nx*ny*nz values
 * each), computed in the handle's arithmetic.  tlbm_create does this itself when params.lbm
 * line 14 is 1, reading the fields from restart_ux.b_dat, restart_uy.b_dat, restart_uz.b_dat
 * and restart_rho.b_dat (raw float32) -- the datasets of the reference's restart.h5, which is
 * HDF5 and is not read here. */
tlbm_status tlbm_load_restart(tlbm_handle* h, const float* ux, const float* uy, const float* uz,
                              const float* rho);

/* ---- post-processing ----------------------------------------------------------------------
 * processTLBM.py (python/processTLBM.py:52-186) on the GPU.  Per node, in global order
 * g = x + y*nx + z*nx*ny and numpy float32 arithmetic (bit-identical to the script on the same
 * float32 inputs): u / (t_conv/l_conv), rho * p_conv - pRef, |u|, F * l_conv/u_conv^2; time
 * averages are first divided by Num_ts.  Output planes, n = nx*ny*nz floats each, in the order
 * of the datasets of hdf5Helper.writeH5 (python/hdf5Helper.py:4-31): ux, uy, uz, |u|, Fx, Fy,
 * Fz, pressure (8 planes); time averages: ux, uy, uz, |u|, pressure (5 planes).  The files are
 * the script's: out{n}.h5 / timeAvg.h5 with its groups and float32 datasets (velo_group,
 * force_group, pres_group; pressure and |u| shaped nz x ny x nx), written without an HDF5
 * library, and data{n}.xmf / timeAvg.xmf, the XDMF of writeXdmf (hdf5Helper.py:58-202). */

/* The processed planes of the last step (time_avg = 0) or of the time-average sums
 * (time_avg = 1, needs params.lbm line 15 = 1) into host memory `out`.  FP64 runs round their
 * values to float32 first. */
tlbm_status tlbm_processed_fields(tlbm_handle* h, int time_avg, float* out);

/* The same, written in the handle's directory: out{k}.h5 + data{k}.xmf for k = 0, 1, ... (one
 * per call, matching the dump numbers when called once per tlbm_write_data), or
 * timeAvg.h5 + timeAvg.xmf.  In-situ: the raw dump files are not needed. */
tlbm_status tlbm_write_processed_data(tlbm_handle* h, int time_avg);

/* Replaces running processTLBM.py in a finished run's directory: reads params.lbm,
 * ordering.b_dat, dumps 0 .. int((Num_ts - Warmup_ts)/plot_freq) - 1 (float32 as the script
 * reads them, or float64 from FP64 runs) and, when line 15 is 1, the time averages; processes
 * them on `device`; writes the files above.  *dumps = dumps processed.  On failure
 * tlbm_get_last_error(NULL) describes it. */
tlbm_status tlbm_process_output_dir(const char* workdir, int device, int* dumps);

/* ---- inflow, learned closure, filtering --------------------------------------------------
 * No counterpart in the reference (its inlet velocity is the scalar uLBM,
 * src/TLBM_Partition.cpp:765-766, and its only closure is Smagorinsky).  Fast arithmetic only. */

/* Inlet velocity u_z per (x, y) of the z = 0 plane: nx*ny values in order x + y*nx (NULL
 * restores the uniform uLBM).  Used for seeded inlet perturbations. */
tlbm_status tlbm_set_inlet_profile(tlbm_handle* h, const double* uz);

/* Learned eddy-viscosity closure for fluid nodes: an 8-32-32-1 MLP (1377 FP32 parameters:
 * W1[32][8], b1[32], W2[32][32], b2[32], w3[32], b3; weights BF16, biases FP32, FP32
 * accumulation, activation tanh of the BF16-rounded pre-activation, in BF16; evaluated on the
 * tensor cores inside the collide kernel) on the normalised features
 * (raw_k - shift[k]) * scale[k] of raw = [Pi_xx, Pi_yy, Pi_zz, Pi_xy, Pi_xz, Pi_yz, rho - 1,
 * |Pi|] (Pi = non-equilibrium stress).  nu_t = max(out_scale * y, nu_smag), nu_smag the
 * reference's Smagorinsky eddy viscosity with params.lbm's cs (no floor when cs = 0), and
 * tau = max(3 (nu + nu_t) + 1/2, tau_min), tau_min > 1/2.  A non-finite output leaves the
 * Smagorinsky rate (plain BGK when cs = 0), which inlet/outlet nodes use too.
 * params = NULL removes the closure. */
tlbm_status tlbm_set_closure_mlp(tlbm_handle* h, const float* params, const float* scale,
                                 const float* shift, float out_scale, float tau_min);

/* Box filter of width `factor` (dividing nx, ny, nz) of the last step's macroscopic fields:
 * writes 10 consecutive coarse fields (rho, ux, uy, uz, ux*ux, uy*uy, uz*uz, ux*uy, ux*uz,
 * uy*uz box means), each (nx/f)*(ny/f)*(nz/f) values of tlbm_output_bytes(h) bytes. */
tlbm_status tlbm_filtered_fields(tlbm_handle* h, int factor, void* out);

/* Training set and optimiser of the learned closure (on the GPU).  Features: n x 8 floats,
 * already normalised; targets: n floats (normalised nu_t).  Loss: mean of (y - t)^2 / 2. */
typedef struct tlbm_mlp tlbm_mlp;
int tlbm_mlp_num_params(void);
tlbm_status tlbm_mlp_create(int64_t n, const float* features, const float* targets,
                            uint64_t seed, int device, tlbm_mlp** out);
tlbm_status tlbm_mlp_destroy(tlbm_mlp* m);
tlbm_status tlbm_mlp_set_params(tlbm_mlp* m, const float* params);
tlbm_status tlbm_mlp_get_params(tlbm_mlp* m, float* params);
/* mean loss and its gradient over samples [first, first+count) in the order given */
tlbm_status tlbm_mlp_loss_grad(tlbm_mlp* m, int64_t first, int64_t count, float* loss,
                               float* grad);
/* Adam (lr; beta 0.9, 0.999) over minibatches of a seeded shuffle; epoch_loss may be NULL */
tlbm_status tlbm_mlp_train(tlbm_mlp* m, int epochs, int64_t batch, float lr, float* epoch_loss);
tlbm_status tlbm_mlp_predict(tlbm_mlp* m, int64_t n, const float* features, float* y);
const char* tlbm_mlp_last_error(const tlbm_mlp* m);

/* ---- batched ensembles ---------------------------------------------------------------------
 * No counterpart in the reference (which runs one channel per job).  `n` independent channels
 * -- each its own tlbm_problem (lattice D3Q15 or D3Q19, size, omega, cs, inlet velocity, outlet
 * density) and node types 0-3 -- advance together: every step is ONE persistent launch over a
 * list of tiles covering all channels, and runs of steps replay a CUDA graph.  Each cell is
 * computed exactly as a single-lattice handle with TLBM_ARITH_FAST computes it, so a channel's
 * fields equal those of a tlbm_handle on the same problem bit for bit.  Storage precision from
 * opt->precision; the arithmetic is always the fast one. */
typedef struct tlbm_ensemble tlbm_ensemble;

tlbm_status tlbm_ensemble_create(int n, const tlbm_problem* problems,
                                 const int32_t* const* nd_types, const tlbm_options* opt,
                                 tlbm_ensemble** out);
tlbm_status tlbm_ensemble_destroy(tlbm_ensemble* e);
/* Tile shape: block_x * block_y threads (block_x a multiple of 32, at most 256 threads), each
 * taking cells_per_thread cells; a tile is that many consecutive cells of one z-plane of one
 * channel, in x-fastest order, so its shape does not depend on the channel's width. */
tlbm_status tlbm_ensemble_set_tiles(tlbm_ensemble* e, int block_x, int block_y,
                                    int cells_per_thread);
/* Times each candidate tile shape over `steps` steps, keeps the fastest, then returns every
 * channel to its initial state; the chosen shape is written to the out-pointers (may be NULL). */
tlbm_status tlbm_ensemble_autotune(tlbm_ensemble* e, int steps, int* block_x, int* block_y,
                                   int* cells_per_thread);
tlbm_status tlbm_ensemble_run(tlbm_ensemble* e, int first_ts, int nsteps);
tlbm_status tlbm_ensemble_time_steps(tlbm_ensemble* e, int first_ts, int nsteps, float* ms);
/* Macroscopic fields of one channel after the last step (global order of that channel). */
tlbm_status tlbm_ensemble_copy_macros(tlbm_ensemble* e, int channel, void* ux, void* uy,
                                      void* uz, void* rho);
tlbm_status tlbm_ensemble_mass(tlbm_ensemble* e, int channel, double* mass);
int64_t tlbm_ensemble_cells(const tlbm_ensemble* e);
int64_t tlbm_ensemble_kernel_launches(const tlbm_ensemble* e);
const char* tlbm_ensemble_last_error(const tlbm_ensemble* e);

/* ---- allocation-free mass reduction --------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory while they
 * run -- applications that reserve the whole GPU for their own memory pool up front, or loops
 * whose policy forbids allocation after start-up -- this computes what tlbm_mass computes, the
 * FP64 sum of all populations, without any allocation: the caller passes the populations
 * (device memory, the engine's layout f[speed * n_cells + cell] in the storage type of
 * `precision`, 16-bit kinds holding f - w) and `mass` (device memory, one double), and the
 * partial sums go to a static device array of 512 KiB that every GPU loading the library keeps
 * until exit.  Limit: n_cells <= 67108864 (65536 partials of 1024 cells); larger inputs return
 * TLBM_ERR_OUT_OF_RANGE and launch nothing.  Each call on a stream that is not being captured
 * looks up that array's address on the current device (make the first call on a device before
 * any stream capture).  Asynchronous on `stream` (a cudaStream_t; NULL is the default stream).
 * All calls share the array: calls that overlap on the GPU race.  The sum is not checked: a
 * diverged run yields NaN or Inf in *mass, not TLBM_ERR_NUMERIC as from tlbm_mass, so test it
 * with isfinite after synchronizing. */
tlbm_status tlbm_mass_static(int q, int precision, int64_t n_cells, const void* populations,
                             double* mass, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TLBM_GB300_H */
