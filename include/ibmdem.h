/*
 * ibmdem.h — C ABI of the GB300 particle-side hot path of IBM-DEM.
 *
 * The reference (zengjs1993/IBM-DEM, Fortran 90 + MPI) exposes this path as
 * argument-less subroutines that act on the module globals `vars` and `ZjsVar`.
 * This header replaces them one-for-one: every reference subroutine on the path
 * has an `ibmdem_<SubroutineName>` entry point acting on a context that owns the
 * device-resident state.  A Fortran caller binds these with ISO_C_BINDING (the
 * record types below are `bind(C)`-compatible mirrors of the reference's derived
 * types); a Python or C caller uses them directly.
 *
 * Conventions
 *   - Every function returns an int status: IBMDEM_OK (0) or a negative error
 *     code; ibmdem_last_error() gives a one-line message for the last failure.
 *   - Host pointers are borrowed for the duration of the call only.
 *   - Work is issued on the context's CUDA stream and is stream-ordered; getters
 *     synchronise that stream before returning.
 *   - One context per host thread; there is no global mutable state.
 *   - Indices in records are 1-based where the reference's are (MSIdx,
 *     globalIdx, localIdx); cell ids are map3Dto1D ids (1-based, Fortran order
 *     over the grid including its 2-cell halo).
 */
#ifndef IBMDEM_H
#define IBMDEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IBMDEM_ABI_VERSION 1

/* status codes */
#define IBMDEM_OK 0
#define IBMDEM_EINVAL (-1)     /* bad argument, size or handle            */
#define IBMDEM_ECUDA (-2)      /* a CUDA runtime call failed              */
#define IBMDEM_ENOMEM (-3)     /* device allocation failed / over budget  */
#define IBMDEM_ERANGE (-4)     /* a parcel left the grid+halo region      */
#define IBMDEM_ECAPACITY (-5)  /* a fixed capacity was exceeded           */
#define IBMDEM_EUNSUPPORTED (-6) /* configuration not supported            */
#define IBMDEM_ESTATE (-7)     /* call out of order (e.g. no lists yet)   */

/* Marker record: mirrors `type Parcel` (ZJS_VARS.F90:6-12) with a fixed
 * C layout (a Fortran shim declares the same fields with bind(C)). 200 bytes. */
typedef struct ibmdem_parcel {
  int32_t globalIdx, localIdx, cellIdx, pType, MSIdx;
  int32_t pad_;
  double radeff, rad, rho, vol, m;
  double x[3], v[3], fcol[3], fdrag[3], vgap[3];
  double wdrag, wsum;
} ibmdem_parcel;

/* Rigid-body record: mirrors `type MultiSphere` (ZJS_VARS.F90:97-102). */
typedef struct ibmdem_multisphere {
  int32_t globalIdx, cpuIdx;
  double rotMat[9], rotMatGlo[9], rotMatGloOld[9], InertiaTensor[9];
  double x[3], xold[3], v[3], vold[3], omega[3], omegaold[3];
  double fcol[3], fmom[3], fdrag[3], AngMom[3], AngMomOld[3];
  double fhydro[3], fmomHydro[3], fmomCol[3];
  double I, rad, rho, vol, m;
} ibmdem_multisphere;

/* Wall collision probe, type WallColProbe (ZJS_VARS.F90:92-94, set up by
 * SetWallProbe, ZJS_INIT_DEM.F90:496-506): a quadrilateral on a solid wall
 * face.  CalculateSolidBoundaryCollisionForce sums the normal spring force
 * n*kn*deltan of every local parcel whose wall contact point lies inside it
 * (WallProbeCollision, ZJS_COLLISION_DEM.F90:150-179), in part order; the sum
 * restarts at every call. */
#define IBMDEM_MAX_WALL_PROBES 60  /* maxNumWallProbe (10) per face, 6 faces */
typedef struct ibmdem_wall_probe {
  int32_t face;          /* 1..6 = -x,+x,-y,+y,-z,+z; the face has bType 1 */
  int32_t pad_;
  double points[4][3];   /* corners in order, points(1:3,1:4)             */
  double force[3];       /* the last call's summed normal force (output)  */
} ibmdem_wall_probe;

/* Case parameters: the reference hard-codes these in source
 * (vars.F90, ZJS_VARS.F90:48-50, ZJS_INIT_DEM.F90:187-194,
 *  initialization.F90:251-259, fluid.F90:257, couplesolverCylinder.F90:12-13). */
typedef struct ibmdem_params {
  int32_t nx, ny, nz;        /* interior cells of the (single-rank) domain   */
  int32_t coupleInterval;    /* DEM sub-steps per fluid step                 */
  int32_t Ns;                /* multi-direct-forcing iterations (ref: 5)     */
  int32_t bType[6];          /* face types -x,+x,-y,+y,-z,+z: 0 = periodic,
                                1 = solid wall; both faces of an axis alike  */
  int32_t pad_;
  double dx, dy, dz;         /* cell sizes                                   */
  double dt;                 /* fluid time step                              */
  double rhof;               /* fluid density                                */
  double knCoeff;            /* spring coefficient                           */
  double ResistCoeff;        /* restitution coefficient e                    */
  double collisionDist;      /* contact distance (ref: 1.5 dx)               */
  double collisionBuffer;    /* list buffer fraction (ref: 0.1)              */
  double gravity[3];         /* (0,0,-9.81) in the reference                 */
} ibmdem_params;

typedef struct ibmdem_ctx ibmdem_ctx;

/* ---- lifetime --------------------------------------------------------- */
/* New context on CUDA device `device`; replaces InitParameters /
 * CopyGridInformationDEM / AllocateDEM / SetCellIndexMapDEM /
 * SetNeighCellIndexForCellsDEM / SetMirrorAndShiftCoords
 * (ZJS_INIT_DEM.F90:67-214) — the tables they build are implicit here. */
int ibmdem_create(const ibmdem_params* p, int32_t device, ibmdem_ctx** out);
int ibmdem_destroy(ibmdem_ctx* ctx);
const char* ibmdem_last_error(const ibmdem_ctx* ctx);
int ibmdem_abi_version(void);
/* Issue work on this CUDA stream (a cudaStream_t passed as void*). */
int ibmdem_set_stream(ibmdem_ctx* ctx, void* stream);
int ibmdem_synchronize(ibmdem_ctx* ctx);

/* ---- state in / out --------------------------------------------------- */
/* Fluid velocity u,v,w in the reference layout: Fortran order
 * (lg1:ug1, lg2:ug2, lg3:ug3), i fastest, 2-cell halo (vars.F90:44,
 * allocate.F90:16-18): (nx+4)*(ny+4)*(nz+4) doubles each.  Also stored as the
 * frozen field that ibmdem_step() restores at the start of every step.
 * Returns when the copies are done.  When the parcels moved since the last
 * spread (new weights), the spread plan for them is built while the fields
 * upload, on a second stream of the same device. */
int ibmdem_set_fluid(ibmdem_ctx* ctx, const double* u, const double* v, const double* w);
/* ibmdem_set_fluid without waiting for the copies: they run on a second stream
 * of the device, component by component, and the forcing loop of
 * ibmdem_MultiDirectForcing starts on each velocity component as soon as that
 * component has arrived.  The caller keeps u,v,w unchanged until the next call
 * that synchronises the context (a getter such as ibmdem_get_bodies, or
 * ibmdem_synchronize). */
int ibmdem_set_fluid_async(ibmdem_ctx* ctx, const double* u, const double* v, const double* w);
/* Copy out u,v,w and the momentum source fx,fy,fz (vars.F90:63), same layout.
 * Any pointer may be NULL. */
int ibmdem_get_fluid(ibmdem_ctx* ctx, double* u, double* v, double* w,
                     double* fx, double* fy, double* fz);
/* ibmdem_get_fluid without waiting: the copies run on `copy_stream` (a
 * cudaStream_t other than the context's), after the work issued so far on the
 * context, and the call returns at once.  Context work that does not write the
 * fields (ibmdem_CloudEvolutionMS) overlaps them; context work that writes the
 * fields waits for them.  Synchronise copy_stream before reading the buffers;
 * they should be pinned for the copies to overlap anything. */
int ibmdem_get_fluid_async(ibmdem_ctx* ctx, double* u, double* v, double* w,
                           double* fx, double* fy, double* fz, void* copy_stream);
/* The read-out of ibmdem_get_fluid_async for a caller that keeps its own copy
 * of the fields, as the Fortran fluid solver does: after MultiDirectForcing the
 * fields differ from what ibmdem_set_fluid loaded only at the nodes the spread
 * touched (and their halo images), and fx,fy,fz are zero elsewhere, so only
 * those nodes' (u, f) pairs are copied -- about 20 bytes per touched node
 * instead of six fields -- and a host thread writes them into u..fz.  u,v,w
 * must hold the field last passed to ibmdem_set_fluid and fx,fy,fz what the
 * previous call left there (zeros before the first); call it after each
 * MultiDirectForcing.  The copies run on copy_stream after the work issued so
 * far and the call returns at once; the arrays are complete when
 * ibmdem_update_fluid_wait returns (ibmdem_set_fluid also waits for them). */
int ibmdem_update_fluid_async(ibmdem_ctx* ctx, double* u, double* v, double* w,
                              double* fx, double* fy, double* fz, void* copy_stream);
int ibmdem_update_fluid_wait(ibmdem_ctx* ctx);
/* Device-to-host bytes of the last completed ibmdem_update_fluid_async. */
int ibmdem_update_fluid_bytes(const ibmdem_ctx* ctx, int64_t* bytes);
/* Local parcels part(1:npLocal) (ZJS_VARS.F90:20); pType is set to -1. */
int ibmdem_set_parcels(ibmdem_ctx* ctx, int32_t np, const ibmdem_parcel* parts);
/* Copy out part(1:np): locals first, then the images, periodic (pType -1) and
 * mirrored across solid walls (pType 1) (np_out gets np,
 * nlocal_out gets npLocal).  cap = capacity of `parts` in records. */
int ibmdem_get_parcels(ibmdem_ctx* ctx, ibmdem_parcel* parts, int32_t cap,
                       int32_t* np_out, int32_t* nlocal_out);
/* Bodies MS(1:nMS) == MSGlo on one rank (ZJS_VARS.F90:106). */
int ibmdem_set_bodies(ibmdem_ctx* ctx, int32_t nMS, const ibmdem_multisphere* ms);
int ibmdem_get_bodies(ibmdem_ctx* ctx, ibmdem_multisphere* ms, int32_t cap, int32_t* nMS_out);

/* ---- list inspection (parity) ----------------------------------------- */
/* Cell lists npPartInCell / partIdxInCell (ZJS_VARS.F90:38-39) as CSR over all
 * ni*nj*nk cells: cell_start[ncell+1] (0-based offsets), items = 1-based part
 * indices.  Pass NULL to query sizes into *ncell_out / *nitems_out. */
int ibmdem_get_cell_lists(ibmdem_ctx* ctx, int32_t* cell_start, int32_t* items,
                          int64_t* ncell_out, int32_t* nitems_out);
/* Contact lists neighPartNo / neighPartIdx (ZJS_VARS.F90:30-31) as CSR over
 * local parcels: start[npLocal+1], idx = 1-based part indices. */
int ibmdem_get_collision_lists(ibmdem_ctx* ctx, int32_t* start, int32_t* idx,
                               int32_t* nlocal_out, int32_t* npairs_out);

/* ---- the hot path: one entry per reference subroutine ----------------- */
/* RebuildParcelInCellListDEM + RebuildParcelCollisionListDEM +
 * RebuildNeighborCellListForParcelsDEM (ZJS_EVOLUTION_DEM.F90:34-41). */
int ibmdem_RebuildAllListOrNot(ibmdem_ctx* ctx);
/* ZJS_UPDATE_LIST_DEM.F90:323-370: delta weights of local parcels. */
int ibmdem_UpdateLocalCellWeightListDEM(ibmdem_ctx* ctx);
/* ZJS_UPDATE_LIST_DEM.F90:372-416: delta weights of the images. */
int ibmdem_UpdateGhostCellWeightListDEM(ibmdem_ctx* ctx);
/* ZJS_UPDATE_LIST_DEM.F90:179-246: refresh image copies (x + shift, v, fdrag;
 * across a wall: x mirrored, the normal v negated, ZJS_MPI_DEM.F90:222-269). */
int ibmdem_UpdateParcelInfoInGhostRegion(ibmdem_ctx* ctx);
/* ZJS_COLLISION_DEM.F90:21-74: spring-dashpot contact force fcol. */
int ibmdem_CalculateCollisionForce(ibmdem_ctx* ctx);
/* Tangential friction of the marker contacts, off while ktRatio == 0 (the
 * default).  No counterpart in the reference, whose contact law is normal only
 * (ZJS_COLLISION_DEM.F90:53-57); with friction off CalculateCollisionForce is
 * the reference's law exactly.  With ktRatio > 0 each touching pair also
 * carries a tangential spring kt = ktRatio*kn with damping
 * etat = eta*sqrt(meff*kt) and a Coulomb limit mu*|fn|: its tangential
 * displacement is kept from one contact-force call to the next, keyed by the
 * parcel ids of both parcels -- a parcel's index in the array last given to
 * ibmdem_set_parcels, which its periodic images share -- so it survives list
 * rebuilds, migrations and periodic images,
 * projected on the new tangent plane and advanced by dtDEM times the tangential
 * relative velocity; beyond the limit the force is scaled to it and the
 * displacement reset to the sliding value.  fcol += n*fn + ft per pair.  The
 * history is dropped by this call and by ibmdem_set_parcels. */
int ibmdem_set_friction(ibmdem_ctx* ctx, double ktRatio, double mu);
/* The tangential history the last contact-force call left, as CSR over the
 * locals: start[nlocal+1], the partner's parcel id per contact (-1: listed but
 * not touching) and 3 displacement components per contact.  Pass NULL to query
 * the sizes.  nlocal is 0 while friction is off. */
int ibmdem_get_friction_history(ibmdem_ctx* ctx, int32_t* start, int32_t* gid, double* xi, int32_t* nlocal_out,
                                int32_t* n_out);
/* ZJS_COLLISION_DEM.F90:76-148: parcel-wall spring-dashpot added to fcol for
 * local parcels in the first or last cell layer, faces -x..+z in order, and the
 * probe sums.  Without walls it does nothing.  The reference also appends a
 * line per probe hit to its log file; this library writes no files. */
int ibmdem_CalculateSolidBoundaryCollisionForce(ibmdem_ctx* ctx);
/* Replace the wall probes (SetWallProbe, ZJS_INIT_DEM.F90:496-506); at most
 * IBMDEM_MAX_WALL_PROBES, each on a face with bType 1, else IBMDEM_EINVAL. */
int ibmdem_set_wall_probes(ibmdem_ctx* ctx, int32_t n, const ibmdem_wall_probe* probes);
/* Copy out the probes with their last force sums (synchronises). */
int ibmdem_get_wall_probes(ibmdem_ctx* ctx, ibmdem_wall_probe* probes, int32_t cap, int32_t* n_out);
/* ZJS_VOLUMEFRACTION_DEM.F90:2-36: interpolation and direct forcing. */
int ibmdem_UpdateFluidVelocityOnLagrangianPoints(ibmdem_ctx* ctx);
/* ZJS_VOLUMEFRACTION_DEM.F90:38-67: deterministic spreading into fx,fy,fz. */
int ibmdem_UpdateMomentumSourceTerm(ibmdem_ctx* ctx);
/* fluid.F90:135-153 + the halo refill of u,v,w (boundary.F90:122-147; beyond a
 * wall the mirrored values negated, boundary.F90:211-245) + Boundary()
 * (fluid.F90:240-249): zero wall-normal velocity on the wall and beyond. */
int ibmdem_VelocityPostGuess(ibmdem_ctx* ctx);
/* ZJS_MS_DEM.F90:494-519 (== AssembleForceMS on one rank, :385-432). */
int ibmdem_AssembleLocalForceMS(ibmdem_ctx* ctx);
/* couplesolverCylinder.F90:2-42 (rigid-body update with Rodrigues rotation). */
int ibmdem_EvolutionMS(ibmdem_ctx* ctx);
/* couplesolverCylinder.F90:44-60 (marker translation, rotation, velocity). */
int ibmdem_ResetVelocityAndPositionLagrangianPoints(ibmdem_ctx* ctx);
/* ZJS_EVOLUTION_DEM.F90:121-150. */
int ibmdem_AdjustParcelPosition(ibmdem_ctx* ctx);

/* ---- fused drivers ---------------------------------------------------- */
/* The list-building tail of InitializationDEM (ZJS_INIT_DEM.F90:24-35). */
int ibmdem_InitializationDEM(ibmdem_ctx* ctx);
/* Particle side of FirstOrderForwardEuler (fluid.F90:252-285): fdrag=0,
 * fx=fy=fz=0, then Ns x {interpolate, image update, spread, post-guess}. */
int ibmdem_MultiDirectForcing(ibmdem_ctx* ctx);
/* couplesolverCylinder.F90:99-187. */
int ibmdem_CloudEvolutionStepMS(ibmdem_ctx* ctx);
/* couplesolverCylinder.F90:189-217. */
int ibmdem_CloudEvolutionMS(ibmdem_ctx* ctx);
/* `nsteps` frozen-fluid steps: restore the fluid set by ibmdem_set_fluid,
 * then ibmdem_MultiDirectForcing + ibmdem_CloudEvolutionMS.  The step's
 * kernels are captured once into a CUDA graph that every step replays (one
 * launch instead of about eighty; captured again when the case's state
 * changes), ordered after the work already on the context's stream and before
 * the work issued on it later; results are the same as issuing the kernels one
 * by one, which happens when step graphs are off, with phase timing on, or
 * when the context's stream is itself being captured. */
int ibmdem_step(ibmdem_ctx* ctx, int32_t nsteps);
/* on = 1 (the default): ibmdem_step replays a captured graph; 0: it issues each
 * kernel on the context's stream.  No counterpart in the reference. */
int ibmdem_set_step_graphs(ibmdem_ctx* ctx, int32_t on);

/* Fluid velocity interpolated at n caller-given points from the context's
 * resident u, v, w: for each point the ulp that
 * ibmdem_UpdateFluidVelocityOnLagrangianPoints forms for a parcel there, same
 * arithmetic.  x: device array of n points (x, y, z), each inside the box
 * [0, nx*dx) x [0, ny*dy) x [0, nz*dz); ulp: device array of n (u, v, w).
 * Allocates nothing: the per-point weights live in a fixed static device array
 * of IBMDEM_PROBE_MAX_POINTS points, and a larger n returns IBMDEM_ERANGE.
 * That array (about 11.3 MB) is part of the library's device module, so every
 * device on which the library's kernels are loaded holds it until the process
 * exits, whether or not this function is ever called.  Each call waits for its
 * result (it synchronises the context's stream), so no call may be made while
 * that stream is being captured into a graph; it returns IBMDEM_ERANGE when a
 * point lies outside the box.  Calls that overlap in time on one device (from
 * several threads or contexts) share that array and race.  No counterpart in
 * the reference. */
#define IBMDEM_PROBE_MAX_POINTS 16384
int ibmdem_interpolate_velocity_noalloc(ibmdem_ctx* ctx, int32_t n, const double* x, double* ulp);

/* ---- unresolved CFD-DEM path ------------------------------------------ */
/* Point particles smaller than a fluid cell (every particle its own body).
 * The reference only holds the drag law of this path (CalculateDragForce,
 * ZJS_DRAGFORCE_DEM.F90:2-35, never called there), a point-particle
 * integrator skeleton (Integration, ZJS_EVOLUTION_DEM.F90:43-75) and an empty
 * LogVolumeFraction (ZJS_EVOLUTION_DEM.F90:27-32); the rest of this path is
 * defined here.  One step:
 *   1. DEM cell lists on a periodic grid of cells >= dcell (stable part order);
 *   2. contacts: for each particle the 27 neighbour cells (k,j,i order,
 *      periodic) in part order; a pair touches when the minimum-image distance
 *      is below rad_i + rad_j.  Normal force as CalculateCollisionForce
 *      (ZJS_COLLISION_DEM.F90:30-57: meff = 2 m_i m_j/(m_i+m_j),
 *      kn = knCoeff/(0.1 dx) meff, etan = eta sqrt(meff kn)); tangential
 *      spring kt = ktRatio kn, etat = eta sqrt(meff kt), Coulomb limit
 *      mu |Fn| with the spring reset to the sliding value; the tangential
 *      displacement of each touching pair is kept per particle across steps
 *      (at most maxContacts partners) and projected on the new tangent plane;
 *   3. solid volume fraction on the fluid cells: each particle spreads its
 *      volume with a Gaussian of sigma = bandwidth * diameter over the 5x5x5
 *      cells around its cell, normalised per particle (weight ((s*gz)*gy)*gx,
 *      s = vol / (sum of the 125 weights * cell volume)); a source cell sums
 *      its particles' weights for one target in part order, and a target sums
 *      those partial sums over the source cells at offsets (dz,dy,dx) in -2..2
 *      (z outermost); alphaf = max(1 - alphap, alphaMin);
 *   4. fluid velocity (trilinear on the MAC faces) and alphaf (trilinear on
 *      the cell centres) at the particle; drag acceleration beta*(u - v) per
 *      component with beta from CalculateDragForce;
 *   5. v += dt*((fdrag + fcol)/m + (1 - rhof/rho) g), omega += dt*tcol/I,
 *      x += dt*v, periodic wrap.
 * The fluid is frozen (the caller owns its solve). */
typedef struct ibmdem_particle {
  int32_t globalIdx, pad_;
  double rad, rho, vol, m, I;    /* radius, density, volume, mass, moment of inertia */
  double x[3], v[3], omega[3];
  double fcol[3], tcol[3];       /* contact force and torque of the last step */
  double fdrag[3];               /* drag force m*beta*(u - v) of the last step */
  double alphaf;                 /* fluid fraction at the particle, last step */
} ibmdem_particle;

typedef struct ibmdem_uparams {
  int32_t nx, ny, nz;            /* fluid cells (cubic, size dx), periodic       */
  int32_t maxContacts;           /* tangential-history partners per particle     */
  double dx;                     /* fluid cell size                              */
  double dcell;                  /* minimum DEM cell size (>= largest diameter)  */
  double dt, rhof, viscf;        /* viscf as ZJS_VARS.F90:77 (1e-5)              */
  double knCoeff, ResistCoeff;   /* normal law as the resolved contacts          */
  double ktRatio, mu;            /* kt = ktRatio*kn (2/7), Coulomb coefficient   */
  double bandwidth;              /* Gaussian sigma = bandwidth * diameter (3)    */
  double alphaMin;               /* lower bound of the fluid fraction            */
  double gravity[3];
} ibmdem_uparams;

typedef struct ibmdem_ucase ibmdem_ucase;
int ibmdem_unresolved_create(const ibmdem_uparams* p, int32_t device, ibmdem_ucase** out);
int ibmdem_unresolved_destroy(ibmdem_ucase* u);
const char* ibmdem_unresolved_last_error(const ibmdem_ucase* u);
int ibmdem_unresolved_set_stream(ibmdem_ucase* u, void* stream);
/* u, v, w as ibmdem_set_fluid: (nx+4)*(ny+4)*(nz+4) doubles, 2-cell periodic halo. */
int ibmdem_unresolved_set_fluid(ibmdem_ucase* u, const double* uf, const double* vf, const double* wf);
int ibmdem_unresolved_set_particles(ibmdem_ucase* u, int32_t n, const ibmdem_particle* parts);
int ibmdem_unresolved_get_particles(ibmdem_ucase* u, ibmdem_particle* parts, int32_t cap, int32_t* n);
/* alphaf of the last step on the nx*ny*nz cells, i fastest. */
int ibmdem_unresolved_get_volume_fraction(ibmdem_ucase* u, double* alphaf);
/* Touching pairs of the last step per particle (CSR over particles, 0-based
 * partner indices) and their tangential displacement (3 doubles each).  Any
 * pointer may be NULL; *ncontacts gets the total. */
int ibmdem_unresolved_get_contacts(ibmdem_ucase* u, int32_t* start, int32_t* partner, double* xi,
                                   int32_t* ncontacts);
int ibmdem_unresolved_step(ibmdem_ucase* u, int32_t nsteps);
int ibmdem_unresolved_synchronize(ibmdem_ucase* u);
int64_t ibmdem_unresolved_launch_count(const ibmdem_ucase* u);
/* Per-phase CUDA-event timing of the unresolved step (lists, search, contacts,
 * stamps, alpha, drag); get_timing synchronises and returns the phase count. */
int ibmdem_unresolved_timing_enable(ibmdem_ucase* u, int32_t on);
int ibmdem_unresolved_get_timing(ibmdem_ucase* u, double* ms, int64_t* counts, int32_t n, int32_t reset);
const char* ibmdem_unresolved_phase_name(int32_t i);
/* CalculateDragForce (ZJS_DRAGFORCE_DEM.F90:2-35) for n particles on device
 * arrays: beta[3i+j] from rho[i], rad[i], v[3i+j], denf, alphaf[i] and the
 * fluid velocity velf[3i+j]; viscf is the reference's 1e-5.  Stream-ordered
 * on `stream`. */
int ibmdem_CalculateDragForce(int32_t n, const double* rho, const double* rad, const double* v, double denf,
                              const double* alphaf, const double* velf, double* beta, void* stream);

/* ---- many cases on one device ---------------------------------------- */
/* Device bytes a case of these parameters, np parcels at the given positions
 * and nMS bodies takes once created and initialised (fields, lists, weights
 * and spread-plan capacities).  No counterpart in the reference. */
int ibmdem_case_bytes(const ibmdem_params* p, int32_t np, const ibmdem_parcel* parts, int32_t nMS, int64_t* bytes);

/* A batch advances many independent cases together: one frozen-fluid step of
 * every member (ibmdem_step) is captured into one CUDA graph whose `lanes`
 * concurrent chains each run a share of the cases, and each batch step is one
 * graph launch.  A case's results are the same in a batch as alone.  Member
 * contexts stay owned by the caller and must be initialised
 * (ibmdem_InitializationDEM) before the first batch step; a member changed
 * outside the batch (new parcels, bodies or lists) is re-captured at the next
 * batch step.  Work on a member's own stream is ordered before and after each
 * ibmdem_batch_step call.  No counterpart in the reference (one case per MPI
 * job there). */
typedef struct ibmdem_batch ibmdem_batch;
int ibmdem_batch_create(int32_t device, ibmdem_batch** out);
int ibmdem_batch_destroy(ibmdem_batch* b);
const char* ibmdem_batch_last_error(const ibmdem_batch* b);
int ibmdem_batch_add(ibmdem_batch* b, ibmdem_ctx* ctx);
/* Number of concurrent chains; 0 = one per case. */
int ibmdem_batch_set_lanes(ibmdem_batch* b, int32_t lanes);
int ibmdem_batch_step(ibmdem_batch* b, int32_t nsteps);
/* Waits for the batch and checks every member for device errors; the first
 * failing member's index goes to *failed_case (-1 if none). */
int ibmdem_batch_synchronize(ibmdem_batch* b, int32_t* failed_case);
/* The forcing loop (the interpolation and the spread of every iteration) of all
 * members in shared launches: fused = 1 gives one interpolation launch
 * (interp_block threads per block, 128 or 256) and one spread launch per
 * iteration for the whole batch, instead of two per member; each member's
 * results are the same.  Members must share Ns (else the batch keeps each
 * member's own launches).  Default: fused = 0, interp_block = 256. */
int ibmdem_batch_set_fused(ibmdem_batch* b, int32_t fused, int32_t interp_block);
int ibmdem_batch_get_config(const ibmdem_batch* b, int32_t* lanes, int32_t* fused, int32_t* interp_block);
/* Times trial_steps batch steps for several lane counts (all, 128, 64, ..., 1)
 * with each member's own forcing launches, then the shared forcing launches
 * (both block sizes) on the two best lane counts, keeps the fastest
 * configuration (ibmdem_batch_get_config) and returns its lane count in
 * *lanes_out.  The trials advance every member. */
int ibmdem_batch_autotune(ibmdem_batch* b, int32_t trial_steps, int32_t* lanes_out);

/* A request server on one device.  Requests wait in a queue (arrival order by
 * default, ibmdem_server_set_policy) and are admitted while the running
 * cases' summed ibmdem_case_bytes stays within
 * hbm_budget and fewer than max_active run.  An admitted case is created on
 * its own stream, initialised, its step captured as a graph and all of its
 * nsteps frozen-fluid steps queued at once, so requests admitted at different
 * times overlap on the device.  ibmdem_server_poll (non-blocking) retires
 * finished cases -- bodies (and parcels when keep_parcels) are read back and
 * the device memory returned -- and admits waiting ones.  The parcel, body and
 * field arrays of a request are borrowed until it leaves the queue; u = v = w =
 * NULL means a fluid at rest.  Latency = completion - submission (host clock).
 * No counterpart in the reference. */
typedef struct ibmdem_server ibmdem_server;
int ibmdem_server_create(int32_t device, int64_t hbm_budget, int32_t max_active, ibmdem_server** out);
int ibmdem_server_destroy(ibmdem_server* s);
const char* ibmdem_server_last_error(const ibmdem_server* s);
int ibmdem_server_submit(ibmdem_server* s, const ibmdem_params* p, int32_t np, const ibmdem_parcel* parts,
                         int32_t nMS, const ibmdem_multisphere* bodies, const double* u, const double* v,
                         const double* w, int32_t nsteps, int32_t keep_parcels, int64_t* id);
/* *pending = requests queued or running. */
int ibmdem_server_poll(ibmdem_server* s, int32_t* pending);
/* *state: 0 queued, 1 running, 2 done, < 0 failed with that status code. */
int ibmdem_server_status(ibmdem_server* s, int64_t id, int32_t* state, double* latency_s, double* queue_s);
int ibmdem_server_result(ibmdem_server* s, int64_t id, ibmdem_parcel* parts, int32_t cap_parts, int32_t* np,
                         int32_t* nlocal, ibmdem_multisphere* bodies, int32_t cap_bodies, int32_t* nMS);
/* Drops a finished request's record and results. */
int ibmdem_server_release(ibmdem_server* s, int64_t id);
int ibmdem_server_memory(const ibmdem_server* s, int64_t* in_use, int64_t* budget);
/* Admit a case only while the running cases hold at most `parcels` markers in
 * total (one case always runs; 0 = no limit): bounds the work that shares the
 * device, so that early requests finish early under load. */
int ibmdem_server_set_work_limit(ibmdem_server* s, int64_t parcels);
/* Admission order: policy 0 = arrival order (the default), 1 = least work first
 * (the queued request with the fewest marker-steps, np * nsteps, that fits),
 * except that once the oldest queued request has waited more than age_limit_s
 * seconds (> 0) the oldest go first again, so no request starves.  Either way
 * a request is admitted only when it fits the budget and the work limit. */
int ibmdem_server_set_policy(ibmdem_server* s, int32_t policy, double age_limit_s);

/* ---- output files ------------------------------------------------------ */
/* OutputCloudTecplot (ZJS_IO_DEM.F90:82-121): the header lines
 * "variables=x,y,z,u,v,w,index,ugap,vgap,wgap" and "zone i=<n> j=1", then per
 * parcel x, v, MSIdx, vgap; with n == 0 one point at `centre` with zeros.  The
 * reference names the file Results/Particle_<trec>_<cpu>.dat. */
int ibmdem_write_tecplot_markers(const char* path, int32_t n, const ibmdem_parcel* parts, const double* centre);
/* The per-body line of fluid.F90:392-397 appended to <dir>/<GlobalIdx>.probe:
 * step, x, v, omega, fdrag/m*rhof, fmom/I*rhof, fcol/m. */
int ibmdem_write_body_probes(const char* dir, int64_t step, int32_t nMS, const ibmdem_multisphere* ms, double rhof);
/* Both files of the context's current state (tecplot_path or probe_dir NULL:
 * that file is skipped).  Device-to-host copies of the local parcels and the
 * bodies run on a stream of the library's own after the work issued so far,
 * later work on the context waits for them, and a host thread formats the files;
 * the call returns at once.  Lines use gfortran's list-directed layout (REAL(8)
 * items as G25.17E3 fields, INTEGER items in 12 columns). */
int ibmdem_output_async(ibmdem_ctx* ctx, const char* tecplot_path, const char* probe_dir, int64_t step);
/* Wait for the files of the last ibmdem_output_async; its status. */
int ibmdem_output_wait(ibmdem_ctx* ctx);

/* ---- fluid stencils (fluid.F90:2-249, boundary.F90:122-247) ----------- */
/* The fluid step of FirstOrderForwardEuler (fluid.F90:251-326) around the
 * Poisson solve, on the context's fields: the particle side's u,v,w and
 * fx,fy,fz and the fields below, all in the layout of ibmdem_set_fluid.  The
 * Poisson solve itself (SetPressureVector, PoissonSolver: PETSc) stays with
 * the caller: it reads the velocity divergence and hands back Pcorr. */
enum {
  IBMDEM_FLUID_U = 0, IBMDEM_FLUID_V, IBMDEM_FLUID_W,
  IBMDEM_FLUID_FX, IBMDEM_FLUID_FY, IBMDEM_FLUID_FZ,
  IBMDEM_FLUID_UOLD, IBMDEM_FLUID_VOLD, IBMDEM_FLUID_WOLD,
  IBMDEM_FLUID_P, IBMDEM_FLUID_PCORR, IBMDEM_FLUID_VELDIV,
  IBMDEM_FLUID_PX, IBMDEM_FLUID_PY, IBMDEM_FLUID_PZ,       /* PressureGradient */
  IBMDEM_FLUID_RHSUL, IBMDEM_FLUID_RHSVL, IBMDEM_FLUID_RHSWL, /* last RHS (Runge-Kutta) */
  IBMDEM_FLUID_OMEGAX, IBMDEM_FLUID_OMEGAY, IBMDEM_FLUID_OMEGAZ,
  IBMDEM_FLUID_NFIELDS
};
/* visc (vars.F90:40) and the constant pressure gradient CPx,CPy,CPz
 * (vars.F90:53) of VelocityGuess's right-hand side. */
int ibmdem_set_fluid_params(ibmdem_ctx* ctx, double visc, double CPx, double CPy, double CPz);
/* One field in or out (host arrays of (nx+4)*(ny+4)*(nz+4) doubles). */
int ibmdem_set_fluid_field(ibmdem_ctx* ctx, int32_t which, const double* a);
int ibmdem_get_fluid_field(ibmdem_ctx* ctx, int32_t which, double* a);
/* uold = u; vold = v; wold = w (fluid.F90:257) */
int ibmdem_StoreOldVelocity(ibmdem_ctx* ctx);
/* VelocityGuess(aRK,bRK,cRK) (fluid.F90:108-133) with ConvectionTensor,
 * ViscousTensor and PressureGradient, bit-identical to the reference's
 * statements; keeps PressureGradient in PX..PZ and the right-hand side in
 * RHSUL..RHSWL. */
int ibmdem_VelocityGuess(ibmdem_ctx* ctx, double aRK, double bRK, double cRK);
/* FillGhostRegionForFluid (boundary.F90:122-147) on one rank for u, v, w, P,
 * omegaZ and Pcorr: periodic copies, or across a solid wall the mirrored
 * layers with u,v,w negated (DealWithBoundaryFluid). */
int ibmdem_FillGhostRegionForFluid(ibmdem_ctx* ctx);
/* Boundary (fluid.F90:240-249): zero wall-normal velocity on and beyond each
 * solid wall. */
int ibmdem_Boundary(ibmdem_ctx* ctx);
/* ModifyBulkVelocity (fluid.F90:155-195) with the switches and targets of
 * DefAveBulk{U,V,W}Switch and bulkU,V,W.  The interior sums are formed in a
 * fixed order of their own (blocks of consecutive nodes, then the blocks in
 * order), not the reference's single running sum: deterministic, and within
 * a few ulps of it. */
int ibmdem_ModifyBulkVelocity(ibmdem_ctx* ctx, int32_t swU, int32_t swV, int32_t swW, double bulkU, double bulkV,
                              double bulkW);
/* VelocityDivergence(cRK) (fluid.F90:93-106) into VELDIV. */
int ibmdem_VelocityDivergence(ibmdem_ctx* ctx, double cRK);
/* PressureCorrection (fluid.F90:197-208): P = P + Pcorr; Pcorr (host, may be
 * NULL to use the PCORR field as it stands) is stored as PCORR first. */
int ibmdem_PressureCorrection(ibmdem_ctx* ctx, const double* Pcorr);
/* VelocityCorrection(cRK) (fluid.F90:210-237), then the vorticity. */
int ibmdem_VelocityCorrection(ibmdem_ctx* ctx, double cRK);
/* SetPressureVector + PoissonSolver + GetLocalArray (poisson.F90:110-186):
 * PCORR on the interior nodes solves the reference's system -- the 7-point
 * Laplacian of SetPressureCorrectionJacobian (poisson.F90:50-108), periodic
 * or Neumann behind a solid wall, with the row of interior node (1,1,1)
 * replaced by PCORR = 0 -- for the right-hand side VELDIV.  Direct FFT solve
 * (FP64), residual far below the reference's KSP tolerance (1e-10).  The
 * halo of PCORR is left as it is.  IBMDEM_EUNSUPPORTED when an extent (doubled
 * along a walled axis) is not a power of two and longer than 2048. */
int ibmdem_PoissonSolver(ibmdem_ctx* ctx);

/* ---- instrumentation -------------------------------------------------- */
/* Record CUDA events around every phase of the drivers (interpolation,
 * spreading, weights, spread plan, cell lists, contact lists, contact force,
 * body sums, body motion, marker motion, image refresh, resets, and the fluid
 * phases: the guess, the halo fills, the other stencils, the Poisson solve). */
int ibmdem_timing_enable(ibmdem_ctx* ctx, int32_t on);
/* Accumulated milliseconds and span counts per phase (synchronises); returns
 * the number of phases.  reset != 0 clears the accumulators. */
int ibmdem_get_timing(ibmdem_ctx* ctx, double* ms, int64_t* counts, int32_t n, int32_t reset);
const char* ibmdem_phase_name(int32_t i);
/* FP64 multiply-add issue rate of `device` in G operations/s (independent
 * chains, best of three launches): the FP64 roofline's denominator. */
int ibmdem_measure_fp64_rate(int32_t device, double* gops);
/* Number of kernel launches this context has issued so far. */
int64_t ibmdem_launch_count(const ibmdem_ctx* ctx);
/* Counters of the current lists: [0]=npLocal [1]=np [2]=pairs
 * [3]=touched u nodes [4]=touched v nodes [5]=touched w nodes
 * [6]=spread contributions.  [3..6] are those of the spread plan the next
 * spread uses; the plan is built here if the weights changed since the last
 * one (a sub-step leaves it to the next spread). */
int ibmdem_get_counters(ibmdem_ctx* ctx, int64_t* out, int32_t n);

#ifdef __cplusplus
}
#endif
#endif /* IBMDEM_H */
