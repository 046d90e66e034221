/*
 * rc_host.h -- host side of the RocketCombustor steady solver for callers that
 * have no Fortran host: it reads a case directory in the reference's own input
 * formats and performs the reference's start-up and set-up, leaving the module
 * arrays that rc_init (rc_gpu.h) takes.
 *
 *   rc_case_open   = startup (src/startup.f90:1) + ReadMesh (src/mesh.f90:2)
 *                    + initialization (src/initialization.f90:1, inlet-width
 *                    rescaling and exit pressure; initial field from fvp1.sav
 *                    through Read_Backup, src/output.f90:276)
 *                    + compute_reconstruction_matrix
 *                    (src/reconstruction_initialization.f90:1)
 *   rc_case_views  = pointers into those arrays, packed as rc_mesh/rc_thermo/rc_config
 *   rc_run_steady  = the steady branch of program main (src/fvm2d.f90:48-150):
 *                    nstep lu_sgs_stage calls with the step_residual norms
 *                    every NScreenOutput steps.
 *
 * Case directory: grid1.in, combustion/{species,thermo,transport,diffusion,
 * chemical_kinetics,oxidizer,fuel}.in, flow/flow_solver_info.in, fvp1.sav.
 */
#ifndef RC_HOST_H
#define RC_HOST_H

#include "rc_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rc_case rc_case;

/* Returns 0 or RC_ERR_ARG; on failure *out is NULL and rc_case_error(NULL)
 * gives the message. */
int rc_case_open(const char* case_dir, rc_case** out);
const char* rc_case_error(const rc_case* c);
void rc_case_close(rc_case* c);

/* Views into the case (valid until rc_case_close).  precision/device fill the
 * two rc_config fields that are not in the case files. */
int rc_case_views(rc_case* c, int precision, int device, rc_mesh* mesh, rc_thermo* thermo, rc_config* cfg);

/* NE, NF, NNT, NVar, Nsp, MaxNei, Nghostcell, nstep_max, NScreenOutput */
void rc_case_dims(const rc_case* c, long* dims);

/* Initial field after initialization: PA(NVar,NE), WA(NVar,NE). */
const double* rc_case_PA(const rc_case* c);
const double* rc_case_WA(const rc_case* c);

/* Named set-up array (same names as the module arrays, e.g. "AMLS", "wdis",
 * "VOL", "Neighbor"); returns a pointer and the element count, or NULL. */
const void* rc_case_array(const rc_case* c, const char* name, long* count);

/* Replace the case's host state (e.g. with what rc_get_state read back). */
int rc_case_set_state(rc_case* c, const double* PA, const double* WA);
/* BackupData (src/output.f90:256): fvp-format restart file of the case's state,
 * readable by Read_Backup (and by rc_case_open); 17 significant digits. */
int rc_case_write_backup(rc_case* c, const char* path, double ttime);
/* output_vtk (src/output.f90:5): legacy ASCII VTK of the cell-centred rho, u,
 * v, p, T, Ma, Y_k and production rates of the case's state. */
int rc_case_write_vtk(rc_case* c, const char* path);

/* Steady driver: rc_init on `device`, nsteps lu_sgs_stage iterations, residual
 * history (step_residual columns Res(1:NVar), romax) written to hist every
 * `every` steps when hist != NULL (hist holds nsteps/every rows), final PA/WA
 * copied back into the case.  Returns the RC status. */
int rc_run_steady(rc_case* c, int precision, int device, long nsteps, long every, double* hist);

/* The same driver for the mixed-precision form with defect correction: runs
 * RC_PREC_MIXED and switches once to RC_PREC_MIXED_DC when the residual
 * (checked every `every` steps) has not dropped below 0.99 times its best
 * value for `window` checks in a row; switched_at gets the switch iteration
 * (0 if it never stalled).  No counterpart in the reference. */
int rc_run_steady_dc(rc_case* c, int device, long nsteps, long every, int window, double* hist, long* switched_at);

/* Time scheme of the case: out[0] 1 for an unsteady scheme (0 steady),
 * ttime, dt, totaltime, nstep_max, InnerLoop, relTol, p_static, A_p, f_p,
 * implicit_time_method (11 values; startup.f90:87-120, initParam.f90:72, the
 * backup's ttime). */
int rc_case_unsteady(const rc_case* c, double* out);

/* Unsteady driver: the implicit branch of program main (src/fvm2d.f90:48-150)
 * with BDF2_stage (src/Time_BDF2.f90:4) or backwardEuler_stage
 * (src/Time_BackwardEuler.f90:4), as the case's implicit_time_method says: up to
 * nsteps physical steps (fewer when totaltime is reached), each advancing
 * ttime, the exit pressure of compute_p_out (fvm2d.f90:229-239) and one
 * rc_bdf2_stage.  inner (may be NULL) gets the inner iterations of each step;
 * hist every `every` steps as in rc_run_steady; the case's state and time
 * advance.  Returns the RC status. */
int rc_run_unsteady(rc_case* c, int device, long nsteps, long every, double* hist, int* inner);

#ifdef __cplusplus
}
#endif
#endif /* RC_HOST_H */
