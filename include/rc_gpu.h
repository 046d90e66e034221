/*
 * rc_gpu.h -- drop-in C ABI for the steady implicit iteration of RocketCombustor
 * (harryzhou2000/RocketCombustor) on one GB300 GPU.
 *
 * The reference runs its hot path as argument-less Fortran subroutines acting
 * on module globals (module mainvar, src/module.f90:2-107).  This ABI keeps
 * those boundaries: the host owns the same arrays in the same Fortran layout
 * (column-major, 1-based indices stored as int32), hands them over once in
 * rc_init, and then calls one entry point per reference subroutine.  The state
 * stays resident on the device between calls; rc_set_state/rc_get_state are the
 * only host<->device copies of the solution.
 *
 * Every entry point returns 0 (RC_OK) or a bit mask of RC_ERR_* codes.  The
 * reference stops the program on these conditions (calls `stop`/MPI_STOP);
 * device-detected conditions are latched in a device error word and reported
 * by the next call that synchronises with the device (rc_residual,
 * rc_get_state, rc_get_array, rc_sync).  rc_last_error() gives a message.
 *
 * Threading: one host thread per context; each context owns one CUDA stream.
 *
 * LU-SGS schedule: by default both sweeps of an iteration run as one
 * cooperative dataflow kernel (per-SM blocks of cells, each pass waiting only
 * for the passes of other blocks that hold its neighbours; FP64 and mixed
 * forms each have theirs); rc_autotune picks the fastest of the schedules,
 * and the environment variable RC_LUSGS_SCHEDULE, read by rc_init, fixes one:
 * "flow", "levels", "levels8", "levels2w", "levels4w" (one kernel per level,
 * with 4 or 8 lanes per cell or, in the FP64 form, each slot's work over two
 * or four warps) or "persistent" (one cooperative kernel with a grid-wide
 * level counter).  All compute the same recurrences bit for bit.
 */
#ifndef RC_GPU_H
#define RC_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define RC_OK 0
#define RC_ERR_THERMO_T 1      /* ComputeGasParameter/compute_enthalpy T out of range (thermo_property.f90:97-101,137-141) */
#define RC_ERR_TRANSPORT_T 2   /* compute_transport_property T out of range (transport_property.f90:101-105) */
#define RC_ERR_NEG_TIMESTEP 4  /* rho, p or T < 0 in TimeStep (TimeStep.f90:66-70) */
#define RC_ERR_NEG_FACE 8      /* rho or p < 0 at a face in flux_lax (flux_lax.f90:239-242) */
#define RC_ERR_NAN 16          /* NaN in WA(1,1) after a stage (Time_LUSGS_steady.f90:24-27) */
#define RC_ERR_BCTYPE 32       /* unknown boundary code (flux_lax.f90:232-235, update_flow_variables.f90:256-259) */
#define RC_ERR_SYNC 64         /* a bounded wait of the cooperative LU-SGS kernels gave up (level counter or pass flag) */
#define RC_ERR_LINSOLVE 128    /* a BDF2 cell system is singular to working precision (dgesvx info /= 0, la_math.f90:176-211) */
#define RC_ERR_ARG 1024        /* invalid argument or unsupported configuration */
#define RC_ERR_CUDA 2048       /* CUDA runtime failure */

#define RC_PREC_FP64 0         /* plain FP64 path, operation order of the reference */
#define RC_PREC_MIXED 1        /* FP32 reconstruction/limiter/flux with compensated accumulation and
                                  FP32 LU-SGS off-diagonal terms; FP64 diagonal, chemistry, Newton, norms */
#define RC_PREC_MIXED_DC 2     /* defect correction: the FP64 residual of RC_PREC_FP64 driving the
                                  FP32 LU-SGS sweeps of RC_PREC_MIXED (FP64 fixed point) */

#define RC_CHEM_EXPLICIT 0     /* chemical source = vol*omega, the reference's explicit rate (sourceterm.f90:43-51) */
#define RC_CHEM_INTEGRATED 1   /* chemical source = vol*rho*(Y(step)-Y)/step from the per-cell integrator */
#define RC_CHEM_SURROGATE 2    /* the same from the learned surrogate (rc_mlp.h), the integrator where the
                                  surrogate's error indicator rejects a cell */

typedef struct rc_ctx rc_ctx;

/*
 * Mesh, geometry and stencils after ReadMesh + compute_reconstruction_matrix,
 * exactly the module arrays of mainvar for one partition (NE_Vir == NE,
 * NF_vir == NF).  Shapes are Fortran shapes; index arrays hold 1-based ids.
 */
typedef struct rc_mesh {
  int NE, NF, NNT, MaxNei, Nghostcell;
  const int* KFace;            /* KFace(NE)                     module.f90:31 */
  const int* Neighbor;         /* Neighbor(2,NF), <0 = -BC code module.f90:28 */
  const int* FNode;            /* FNode(2,NF)                   module.f90:28 */
  const int* FProperty;        /* FProperty(NF)                 module.f90:28 */
  const int* NeighF;           /* NeighF(4,NE), ascending face  module.f90:31 */
  const int* Neigh;            /* Neigh(NE)                     module.f90:31 */
  const int* NeighC;           /* NeighC(0:MaxNei,NE)           module.f90:31 */
  const int* Ghostcell;        /* Ghostcell(MaxNei,NE)          module.f90:46 */
  const int* Num_ghostcell;    /* Num_ghostcell(NE)             module.f90:46 */
  const int* Hostcell;         /* Hostcell(Nghostcell)          module.f90:46 */
  const int* BCtype_Ghostcell; /* BCtype_Ghostcell(Nghostcell)  module.f90:46 */
  const double* COOR;          /* COOR(2,NNT)                   module.f90:38 */
  const double* VECX;          /* VECX(2,NF)                    module.f90:40 */
  const double* SideOfs;       /* SideOfs(2,NF)                 module.f90:40 */
  const double* VOL;           /* VOL(NE)                       module.f90:42 */
  const double* CELLXY;        /* CELLXY(2,NE)                  module.f90:42 */
  const double* reflen;        /* reflen(2,NE)                  module.f90:42 */
  const double* wdis;          /* wdis(MaxNei,NE)               module.f90:51 */
  const double* AMLS;          /* AMLS(2,MaxNei,NE)             module.f90:67 */
  const double* Coor_Ghostnode;/* Coor_Ghostnode(2,4,Nghostcell) module.f90:47 */
  double total_volume;         /* total_volume                  module.f90:36 */
} rc_mesh;

/*
 * Species, thermo, transport, diffusion, kinetics and inlet data as held by the
 * modules of src/combustion_modeling after start-up and initialization (the
 * inlet mass flows already divided by the inlet widths, initialization.f90:19-23).
 */
typedef struct rc_thermo {
  int Nsp;                              /* species.f90:7 */
  double Rconstant;                     /* species.f90:8 */
  const double* mole_weight;            /* (Nsp) */
  const double* R_species;              /* (Nsp) */
  int order_of_cp_polynomial;           /* thermo_property.f90:86, must be 7 */
  double thermo_lowest_tem, thermo_critical_tem, thermo_highest_tem;
  const double* low_coef_Cp_species;    /* (order,Nsp) */
  const double* high_coef_Cp_species;   /* (order,Nsp) */
  const double* low_enthalpy_b1;        /* (Nsp) */
  const double* high_enthalpy_b1;       /* (Nsp) */
  double transport_lowest_tem, transport_critical_tem, transport_highest_tem;
  const double* mu_K[16];               /* low_mu_A..D, high_mu_A..D, low_K_A..D, high_K_A..D, each (Nsp) */
  const double* collision_diameter;     /* (Nsp) diffusion_velocity.f90:7 */
  const double* LJ_energy;              /* (Nsp) */
  int code_chemical_model;              /* chemical_kinetics.f90:6 */
  const double* coef_f_react;           /* (Nsp) of reaction 1 */
  const double* coef_r_react;           /* (Nsp) of reaction 1 */
  double Af_react, E_react;             /* reaction 1 */
  const double* oxidizer_mass_fraction; /* (Nsp) oxidizer.f90:9 */
  double oxidizer_temp_in, oxidizer_mass_flow;
  const double* fuel_mass_fraction;     /* (Nsp) fuel.f90:9 */
  double fuel_temp_in, fuel_mass_flow;
} rc_thermo;

/* Solver flags read by startup (startup.f90:55-128) that select the path. */
typedef struct rc_config {
  int IfViscous;
  int If_turn_on_combustion;
  int limit_ID;
  double cfl;
  double p_out;      /* exit pressure, initialization.f90:32-33 */
  int precision;     /* RC_PREC_* */
  int device;        /* CUDA device ordinal */
} rc_config;

/* Upload geometry, stencils and tables; build the device layout and the
 * LU-SGS level schedule from the reference cell order.
 * Replaces the state left by ReadMesh/compute_reconstruction_matrix
 * (src/mesh.f90:2, src/reconstruction_initialization.f90:1). */
int rc_init(const rc_mesh* mesh, const rc_thermo* thermo, const rc_config* cfg, rc_ctx** out);
int rc_finalize(rc_ctx* ctx);

/* A batch of ncase independent cases in one context (one launch per kernel
 * for all of them): meshes[k], thermos[k], cfgs[k] describe case k as rc_init
 * takes them.  Gas data and solver flags must agree; inlets and p_out may
 * differ.  The cases are renumbered into one mesh, case k's cells following
 * those of cases 0..k-1; states (rc_set_state/rc_get_state, rc_get_array) use
 * that numbering, i.e. the cases' Fortran arrays concatenated.  Each case runs
 * the recurrences it runs alone (the LU-SGS levels never mix cases), so its
 * results are bit-identical to a single-case context.  No counterpart in the
 * reference (one case per run). */
int rc_init_batch(int ncase, const rc_mesh* meshes, const rc_thermo* thermos, const rc_config* cfgs, rc_ctx** out);
/* Number of cases and the ncase+1 cell offsets of the numbering. */
int rc_batch_info(rc_ctx* ctx, int* ncase, int* cell_offsets);

/* PA(NVar,NE), WA(NVar,NE) in the Fortran layout (module.f90:54).  Either
 * pointer may be null.  Page-locked host buffers (cudaHostAlloc,
 * cudaHostRegister) are read and written in place by the device's layout
 * kernel; pageable ones go through one copy.  rc_set_state queues its work on
 * the context's stream and returns: from page-locked memory the device may
 * still be reading, so the caller keeps such buffers unchanged until its next
 * call that synchronises (rc_get_state, rc_residual, rc_sync).  rc_get_state
 * returns when both arrays are on the host. */
int rc_set_state(rc_ctx* ctx, const double* PA, const double* WA);
int rc_get_state(rc_ctx* ctx, double* PA, double* WA);

/* One entry point per reference subroutine, acting on device-resident state. */
int rc_timestep(rc_ctx* ctx);          /* TimeStep            TimeStep.f90:4 */
int rc_reconstruction(rc_ctx* ctx);    /* reconstruction      fvm2d.f90:183 (gradient + Limiter_Barth) */
int rc_flux_sourceterm(rc_ctx* ctx);   /* flux_sourceterm     fvm2d.f90:196 (flux_lax + flux_viscous + sourceterm) */
int rc_lusgs_steady(rc_ctx* ctx);      /* LU_SGS_steady       Time_LUSGS_steady.f90:32 (incl. update_primitve_variables) */
int rc_lusgs_stage(rc_ctx* ctx, int istep); /* lu_sgs_stage   Time_LUSGS_steady.f90:4, one captured graph */

/* Switch the precision of the following calls: RC_PREC_FP64 on any context,
 * RC_PREC_MIXED / RC_PREC_MIXED_DC on contexts created with a mixed mode.  A
 * driver switches MIXED -> MIXED_DC when the FP32 residual stops decreasing.
 * No counterpart in the reference (it has a single FP64 path). */
int rc_set_precision(rc_ctx* ctx, int precision);

/* Polls after which a level wait of the persistent LU-SGS kernels gives up
 * (default 2^24): the kernel then latches RC_ERR_SYNC and returns, leaving the
 * context usable.  A small limit forces the timeout path (fault tests).  The
 * Newton-update warps of the mixed forms' dataflow launch wait through the
 * whole forward sweep with polls at least 256 ns apart and count them against
 * the same limit, so a limit set by hand must cover the forward sweep's
 * duration divided by 256 ns (the default covers over 4 s). */
int rc_set_wait_limit(rc_ctx* ctx, unsigned polls);
/* Clear the latched stop conditions (after the caller has dealt with them). */
int rc_clear_error(rc_ctx* ctx);

/* Host-only check of the dataflow LU-SGS plan that rc_init builds for the
 * cell graph (no device work; callable without a GPU).  nface[i] <= 4 faces of
 * cell i, cother[q*ne + i] the cell across face q (-1 at a boundary), nblocks
 * blocks.  Checks that every cell is in exactly one pass of each sweep, that a
 * pass's dependencies are passes of other blocks at lower levels and cover
 * every neighbour it reads from another block, and runs the blocks' protocol
 * in synchronous steps (each block finishes its next pass once its
 * dependencies are done) to the end.  stats[8]: forward passes, backward
 * passes, dependencies, most dependencies of one pass, steps, forward levels,
 * backward levels, cells per block.  Returns RC_OK, RC_ERR_ARG (bad input) or
 * RC_ERR_SYNC (a check failed or the steps stalled). */
int rc_flow_plan_check(int ne, int nblocks, const int* nface, const int* cother, long long* stats);
/* The same checks and stats for one plan: passes of `groups` groups of 8
 * positions (compact = 0; groups 1..3) or the compact plan of `groups` groups
 * (compact = 1; groups 1..2) of at most min(128 / nvar, 32) cells and 32
 * active (cell, face) pairs each, for which it also checks that each group
 * lists exactly its cells' active pairs.  Host only, like rc_flow_plan_check. */
int rc_flow_plan_stats(int ne, int nblocks, const int* nface, const int* cother, int groups, int compact, int nvar,
                       long long* stats);

/* Autotuner: times `iters` iterations of every launch configuration (LU-SGS
 * as one cooperative kernel, one kernel per level or, in the FP64 form, the
 * dataflow kernel; 64 or 128 threads per block for the cell and face kernels)
 * on the current state, keeps the
 * fastest and restores the state.  The configurations compute the same bits.
 * report (may be null) gets one line of timings.  Synchronises. */
int rc_autotune(rc_ctx* ctx, int iters, char* report, int report_len);

/* Chemistry source of the following iterations (all precision modes; the
 * chemistry is FP64 in each).  RC_CHEM_INTEGRATED integrates each cell's
 * constant-volume adiabatic reactor over its pseudo time step with linearly
 * implicit substeps built on Compute_Con_to_Pri_Jaco (Con_to_Pri_Jacobian.f90:1)
 * and compute_derivative_production_rate (chemical_kinetics.f90:167); tol is
 * the relative change allowed per substep (0.05 by default), max_substeps the
 * cap (200).  The reference has no such integrator: it is new.  Needs
 * If_turn_on_combustion. */
int rc_set_chemistry(rc_ctx* ctx, int mode, double tol, int max_substeps);
/* Accepted substeps per cell of the last integrated source (NE ints, host);
 * zeros before the first one.  Synchronises. */
int rc_chem_substeps(rc_ctx* ctx, int* nsub);
/* Integrate n primitive states over their own dt with the same integrator:
 * d_P and d_out are DEVICE arrays in SoA layout (component k of state i at
 * [k*n + i], NVar components), d_dt and d_nsub device arrays of n.  Runs on the
 * context's stream; stop conditions latch like the other calls. */
int rc_chem_integrate(rc_ctx* ctx, const double* d_P, const double* d_dt, int n, double* d_out, int* d_nsub,
                      double tol, int max_substeps);

/* Learned surrogate of the integrator (needs Nsp = 4).  The network (rc_mlp.h)
 * is owned by the caller and must outlive its use.  A cell goes back to the
 * integrator when its state is outside the network's training domain, when
 * the predicted normalised changes of the reacting species differ by more than
 * spread_tol, or when the prediction leaves Y in [0, 1]. */
struct rc_mlp;
int rc_set_surrogate(rc_ctx* ctx, struct rc_mlp* net, double spread_tol);
/* Cells of the last surrogate source served by the network / by the integrator. */
int rc_surrogate_stats(rc_ctx* ctx, unsigned* n_surrogate, unsigned* n_fallback);
/* Freeze (on != 0) or free (on = 0) the surrogate's per-cell choice between
 * the network and the integrator.  With on, the next rc_lusgs_stage records
 * every cell's choice and the stages after it keep it (a network cell whose
 * source is not finite still goes to the integrator): the source is then a
 * smooth function of the state, which a steady iteration needs to converge
 * (the choice itself switches as the state moves near a threshold).  No
 * counterpart in the reference.  Returns RC_ERR_ARG before rc_set_surrogate. */
int rc_surrogate_freeze(rc_ctx* ctx, int on);
/* Training pairs from integrated states: d_P0, d_P1 (NVar x n SoA, before and
 * after d_dt) -> raw features d_x (n x 7: T, p, Y_1..Y_4, dt) and targets d_t
 * (n x 4: the normalised changes z_k of rc_mlp.h).  Device pointers; on the
 * context's stream. */
int rc_surrogate_samples(rc_ctx* ctx, const double* d_P0, const double* d_P1, const double* d_dt, int n, float* d_x,
                         float* d_t);

/*
 * Unsteady dual-time BDF2 (implicit_time_method 5): the reference's shipped
 * time scheme.  One context, one case, FP64, explicit chemical source.
 *
 * rc_set_p_out replaces the exit pressure of each case (ncase values) for the
 * following calls: the host's compute_p_out (fvm2d.f90:229-239) result at the
 * current time.
 *
 * rc_bdf2_stage = BDF2_stage (Time_BDF2.f90:4-69): shifts the time levels
 * (istep 1: WP = WP2 = WA, phi = 0; later WP2 = WP, WP = WA, phi = 1/2), then
 * up to inner_loop inner iterations of timestep, reconstruction,
 * flux_sourceterm and BDF2_LU_SGS, each one CUDA graph launch, stopped when
 * the species rows of the normalised residual of the primitive increments
 * drop below rel_tol times their value at the first inner iteration
 * (inner_iteration_residual, residual.f90:23-59), and ends with one more
 * reconstruction and flux_sourceterm.  dt is the physical time step (the
 * driver shortens the last one, fvm2d.f90:52-56).  *inner_done gets the inner
 * iterations taken.  Synchronises once per inner iteration.
 *
 * rc_bdf2_lusgs = BDF2_LU_SGS (Time_BDF2.f90:71-337) alone, for per-subroutine
 * checks: on inner_rk 1 the source term vol/dt ((1+2 phi) WP - phi WP2) is
 * formed from the time levels "WP" and "WP2" (rc_set_array), then the
 * primitive-variable LU-SGS sweeps with the per-cell 7x7 solves of
 * advanced_linear_solve_lapack (la_math.f90:120-213) and the update of PA and
 * WA.  A cell system singular to working precision latches RC_ERR_LINSOLVE
 * (the reference stops).
 */
int rc_set_p_out(rc_ctx* ctx, const double* p_out);
int rc_bdf2_stage(rc_ctx* ctx, int istep, double dt, int inner_loop, double rel_tol, int* inner_done);
int rc_bdf2_lusgs(rc_ctx* ctx, int inner_rk, double phi, double dt);
/* Backward Euler (implicit_time_method 3): backwardEuler_stage and
 * backwardEuler_LU_SGS (Time_BackwardEuler.f90:4-324).  The same sweeps,
 * per-cell solves and inner-iteration stop as BDF2; the source term is
 * vol/dt WA at the first inner iteration, the diagonal and right-hand side
 * those of phi = 0, and there are no time levels. */
int rc_euler_stage(rc_ctx* ctx, int istep, double dt, int inner_loop, double rel_tol, int* inner_done);
int rc_euler_lusgs(rc_ctx* ctx, int inner_rk, double dt);

/* Residual + step_residual norms (residual.f90:4-21, 61-79): res(k) =
 * sum(vol*|hWA(k,:)|)/total_volume, romax = max(WA(1,:)).  Synchronises. */
int rc_residual(rc_ctx* ctx, double* res, double* romax);
/* The same norms per case of a batch: res(NVar, ncase), romax(ncase).  A case
 * gets the bits it gets alone.  Synchronises. */
int rc_residual_batch(rc_ctx* ctx, double* res, double* romax);

/* Wait for queued work; returns the latched device error bits. */
int rc_sync(rc_ctx* ctx);

/* Intermediate arrays in the Fortran layout, for per-subroutine checks:
 * "PA","WA","hWA" (NVar,NE); "GradC" (2,NVar,NE); "alpaF" (NF); "step" (NE);
 * "GPA" (NVar,Nghostcell); "WP", "WP2" (NVar,NE), the BDF2 time levels.
 * rc_set_array accepts the same names. */
int rc_get_array(rc_ctx* ctx, const char* name, double* out);
int rc_set_array(rc_ctx* ctx, const char* name, const double* in);

/* Run all work of this context on a caller-provided cudaStream_t. */
int rc_set_stream(rc_ctx* ctx, void* cuda_stream);
void* rc_get_stream(rc_ctx* ctx);

/* Kernel launches issued by this context so far (graph replays counted per
 * captured kernel node) and the number of LU-SGS levels of each sweep. */
int rc_stats(rc_ctx* ctx, long long* kernel_launches, int* fwd_levels, int* bwd_levels);

/* Measured FP64 rate of the current device (no counterpart in the reference:
 * a measurement aid).  A kernel of 8 independent DADD/DMUL chains per thread,
 * 8 blocks of 256 threads per SM, `iters` steps of each chain, timed with CUDA
 * events on cuda_stream after one shorter warm-up launch.  ops_per_s =
 * thread-level FP64 operations per second; seconds = the timed launch. */
int rc_fp64_rate(void* cuda_stream, int iters, double* ops_per_s, double* seconds);

const char* rc_last_error(rc_ctx* ctx);

/* The same message copied into a caller buffer of len bytes, the form a
 * Fortran host binds (character(kind=c_char) :: buf(len)) to print it before
 * MPI_STOP (src/parallel.f90:56-62 stops with a message).  At most len-1
 * bytes of the message are copied and a NUL always follows them.  Returns
 * RC_OK, or RC_ERR_ARG when buf is NULL or len < 1 (nothing written). */
int rc_last_error_buf(rc_ctx* ctx, char* buf, int len);

/*
 * Residual norms of device arrays that the caller owns, computed without any
 * device allocation.  No counterpart in the reference: it serves hosts that
 * cannot call cudaMalloc, such as a Fortran host whose device arrays are all
 * managed by its own CUDA Fortran/OpenACC runtime, or a solver loop that must
 * not allocate (cudaMalloc can synchronise the whole device) once it is set up.
 *
 * Inputs: d_hWA and d_WA in the Fortran layout (NVar,NE) and d_VOL (NE), all in
 * device memory of the current device; the result is the same as rc_residual:
 * res(k) = sum(VOL*|hWA(k,:)|)/total_volume, romax = max(WA(1,:)), written to
 * host memory.  The work runs on cuda_stream (NULL = legacy default stream) and
 * the call returns after it has finished.
 *
 * Scratch: a fixed array compiled into the library, sized for NVar up to
 * RC_NOALLOC_MAX_NVAR (about 41 KB, held by every GPU that loads the library
 * until the process exits); a larger NVar is rejected with RC_ERR_ARG and a
 * message on stderr.  Every call looks up the array's device address
 * (cudaGetSymbolAddress) in the device and context current on the calling
 * thread, so the address stays right after cudaDeviceReset and under a
 * non-primary context; the first call on a device may load the module, so make
 * it before any stream capture.  Every value read from the scratch is written
 * earlier in the same call, so nothing has to be cleared between calls, but all
 * calls share the one array: calls whose work overlaps on the GPU (other
 * streams, other host threads) race and must be serialised by the caller.
 */
#define RC_NOALLOC_MAX_NVAR 16
int rc_residual_noalloc(const double* d_hWA, const double* d_WA, const double* d_VOL, int NE, int NVar,
                        double total_volume, void* cuda_stream, double* res, double* romax);

#ifdef __cplusplus
}
#endif
#endif /* RC_GPU_H */
