/*
 * ibmdem_oracle.h — CPU restatement of the IBM-DEM particle-side hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity reference for the GPU
 * library (libibmdem) and the timed CPU baseline; nothing in the product links
 * or calls it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs
 * load it.
 *
 * PARITY PINNED to the reference's own subroutines: the reference (Fortran 90
 * + MPI + PETSc) cannot be compiled here and ships no tests or golden vectors,
 * so tests/golden/fortran_subset.py runs its Fortran statements through a
 * translator on one rank, and tests/test_reference_pins.py checks this
 * restatement against what they produce (tests/golden/ref_*.npz), bit for bit
 * at every stage of two coupled cases.  The restatement follows the reference
 * source line by line (file:line cited at each function); analytic checks
 * (tests/test_oracle_*.py) cover what the reference does not have.
 *
 * The entry points mirror the reference subroutines one-for-one and operate on
 * one single-rank case, each axis periodic or between two solid walls.  Record layouts are the C-ABI ones
 * from include/ibmdem.h.
 */
#ifndef IBMDEM_ORACLE_H
#define IBMDEM_ORACLE_H
#include "../include/ibmdem.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_case orc_case;

orc_case* orc_create(const ibmdem_params* p);
void orc_destroy(orc_case* c);
const char* orc_last_error(const orc_case* c);
void orc_set_threads(int n);
int orc_get_threads(void);

int orc_set_fluid(orc_case* c, const double* u, const double* v, const double* w);
int orc_get_fluid(orc_case* c, double* u, double* v, double* w, double* fx, double* fy, double* fz);
int orc_set_parcels(orc_case* c, int32_t np, const ibmdem_parcel* parts);
int orc_get_parcels(orc_case* c, ibmdem_parcel* parts, int32_t cap, int32_t* np_out, int32_t* nlocal_out);
int orc_set_bodies(orc_case* c, int32_t n, const ibmdem_multisphere* ms);
int orc_get_bodies(orc_case* c, ibmdem_multisphere* ms, int32_t cap, int32_t* n_out);
int orc_get_cell_lists(orc_case* c, int32_t* cell_start, int32_t* items, int64_t* ncell_out, int32_t* nitems_out);
int orc_get_collision_lists(orc_case* c, int32_t* start, int32_t* idx, int32_t* nlocal_out, int32_t* npairs_out);
/* Per-marker delta weights of the 125 stencil cells (3 components), for the
 * first `n` parcels: w[(p*125 + j)*3 + comp]; cells[p*125 + j] (0 = absent). */
int orc_get_weights(orc_case* c, int32_t n, double* w, int32_t* cells);

int orc_RebuildAllListOrNot(orc_case* c);
int orc_UpdateLocalCellWeightListDEM(orc_case* c);
int orc_UpdateGhostCellWeightListDEM(orc_case* c);
int orc_UpdateParcelInfoInGhostRegion(orc_case* c);
int orc_CalculateCollisionForce(orc_case* c);
/* tangential friction of the marker contacts, off while ktRatio == 0 (not in
 * the reference); drops the tangential history */
int orc_set_friction(orc_case* c, double ktRatio, double mu);
int orc_get_friction_history(orc_case* c, int32_t* start, int32_t* gid, double* xi, int32_t* nl_out,
                             int32_t* n_out);
int orc_CalculateSolidBoundaryCollisionForce(orc_case* c);
int orc_set_wall_probes(orc_case* c, int32_t n, const ibmdem_wall_probe* probes);
int orc_get_wall_probes(orc_case* c, ibmdem_wall_probe* probes, int32_t cap, int32_t* n_out);
int orc_UpdateFluidVelocityOnLagrangianPoints(orc_case* c);
int orc_UpdateMomentumSourceTerm(orc_case* c);
int orc_VelocityPostGuess(orc_case* c);
int orc_AssembleLocalForceMS(orc_case* c);
int orc_EvolutionMS(orc_case* c);
int orc_ResetVelocityAndPositionLagrangianPoints(orc_case* c);
int orc_AdjustParcelPosition(orc_case* c);

int orc_InitializationDEM(orc_case* c);
int orc_MultiDirectForcing(orc_case* c);
int orc_CloudEvolutionStepMS(orc_case* c);
int orc_CloudEvolutionMS(orc_case* c);
int orc_step(orc_case* c, int32_t nsteps);

/* Drag coefficient of ZJS_DRAGFORCE_DEM.F90:2-35 for one parcel. */
void orc_CalculateDragForce(double rho_p, double rad_p, const double* v_p, double denf,
                            double alphaf_local, const double* velf, double* beta);
/* eta of ZJS_COLLISION_DEM.F90:30 (single-precision pi literal reproduced). */
double orc_eta(double ResistCoeff);

/* Unresolved CFD-DEM path (unresolved_oracle.c): the definition in
 * include/ibmdem.h, same loop and evaluation order as the CUDA path. */
typedef struct orc_ucase orc_ucase;
orc_ucase* orc_u_create(const ibmdem_uparams* p);
void orc_u_destroy(orc_ucase* u);
const char* orc_u_last_error(const orc_ucase* u);
int orc_u_set_fluid(orc_ucase* u, const double* uf, const double* vf, const double* wf);
int orc_u_set_particles(orc_ucase* u, int32_t np, const ibmdem_particle* parts);
int orc_u_get_particles(orc_ucase* u, ibmdem_particle* parts, int32_t cap, int32_t* n);
int orc_u_get_volume_fraction(orc_ucase* u, double* alphaf);
int orc_u_get_contacts(orc_ucase* u, int32_t* start, int32_t* partner, double* xi, int32_t* ncontacts);
int orc_u_step(orc_ucase* u, int32_t nsteps);

/* fluid stencils (fluid_oracle.c) */
typedef struct orc_fluid orc_fluid;
orc_fluid* orc_fluid_create(const ibmdem_params* p);
void orc_fluid_destroy(orc_fluid* F);
void orc_fluid_set_params(orc_fluid* F, double visc, double CPx, double CPy, double CPz);
int orc_fluid_set_field(orc_fluid* F, int which, const double* a);
int orc_fluid_get_field(orc_fluid* F, int which, double* a);
void orc_fluid_StoreOldVelocity(orc_fluid* F);
void orc_fluid_VelocityGuess(orc_fluid* F, double aRK, double bRK, double cRK);
void orc_fluid_FillGhostRegionForFluid(orc_fluid* F);
void orc_fluid_Boundary(orc_fluid* F);
void orc_fluid_ModifyBulkVelocity(orc_fluid* F, int swU, int swV, int swW, double bulkU, double bulkV, double bulkW);
void orc_fluid_VelocityDivergence(orc_fluid* F, double cRK);
void orc_fluid_PressureCorrection(orc_fluid* F);
void orc_fluid_VelocityCorrection(orc_fluid* F, double cRK);
void orc_fluid_PressureOperator(orc_fluid* F, const double* p, double* out);

#ifdef __cplusplus
}
#endif
#endif
