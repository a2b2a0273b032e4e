/*
 * ibmdem_oracle.c — CPU restatement of the IBM-DEM particle-side hot path.
 *
 * TEST INFRASTRUCTURE ONLY (parity reference and timed CPU baseline); the
 * product never links or calls it.  PARITY PINNED: the Fortran reference
 * cannot be compiled here and has no tests or golden vectors for this path;
 * this file restates its source, citing file:line for each routine, and
 * agrees bit for bit with the reference's own subroutines run through the
 * Fortran-subset translator of tests/golden/fortran_subset.py
 * (tests/test_reference_pins.py), besides the analytic checks in
 * tests/test_oracle_*.py.
 *
 * Scope: one MPI rank owning the whole domain; each axis either periodic
 * (bType = 0 on both faces) or bounded by two solid walls (bType = 1).  On one
 * rank the reference's MPI_SENDRECV calls for periodic faces send to the rank
 * itself; they are restated as the copies they perform.  A wall face has no
 * neighbour rank (neighCpu = -1), so the reference takes its
 * UpdateFullInfoForSolidOutletBoundary / UpdatePartInfoForSolidOutletBoundary
 * and DealWithBoundaryFluid branches there.
 *
 * Floating point: compile with -ffp-contract=off (gfortran on x86-64 without
 * -march emits no FMA).  Every expression keeps the Fortran left-to-right
 * evaluation order, integer literals are exact doubles, and the one
 * single-precision literal on the path (3.1415926536**2 in eta) is reproduced.
 *
 * Deliberate deviations, all documented at the routine they touch:
 *  1. Multi-rank body semantics: every body is integrated (the one-rank branch
 *     at couplesolverCylinder.F90:114-121 forces nMSlocal = 1).
 *  2. Body-relative marker vectors use the periodic image of the body centre
 *     nearest the marker (AssembleLocalForceMS, ResetVelocityAndPosition...):
 *     the one-rank reference uses the raw difference, which is off by a box
 *     length for a body straddling a periodic face.  Identical otherwise.
 *  3. Capacities are dynamic (maxPartNo, maxCollisionNo, maxPartNoInCell are
 *     unchecked fixed arrays in the reference); the cell lists are stored as
 *     CSR with the reference's per-cell insertion order.
 *  4. Halo cells of fx,fy,fz (accumulated and then discarded by the reference)
 *     are not part of the state: VelocityPostGuess reads interior cells only.
 *  5. A periodic image receives only the fields MyMPISendAndRecv sends; its
 *     vgap and wdrag keep whatever the slot held before in the reference.  Here
 *     they are zero, so that a marker that migrates across a periodic face (its
 *     image becomes the local) has a defined vgap until the next interpolation.
 */
#include "ibmdem_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef ibmdem_parcel Parcel;
typedef ibmdem_multisphere MultiSphere;

#define NST 125 /* maxNeighCellNo (ZJS_VARS.F90:5) */
#define HALO 2  /* haloX/Y/Z (ZJS_VARS.F90:68) and lap (vars.F90:14) */

struct orc_case {
  ibmdem_params p;
  int n[3];
  int SG[3], EG[3], LG[3], UG[3];
  int ni, nj, nk;
  int64_t ncell;
  double di, dj, dk;
  double start[3], end[3], len[3];
  double coordShift[6];
  double coordMirror[6]; /* wall coordinates (ZJS_INIT_DEM.F90:145-150) */
  double pointBound[6][3], normBound[6][3]; /* wall planes (ZJS_INIT_DEM.F90:120-137) */
  /* wall probes (type WallColProbe, ZJS_VARS.F90:92-94), in the caller's order */
  int nProbe;
  ibmdem_wall_probe probe[IBMDEM_MAX_WALL_PROBES];
  double dtDEM, eta, cut2;
  /* parcels part(1:np); locals are part(1:npLocal) */
  Parcel* part;
  int np, npLocal, cap;
  /* bodies MS == MSGlo on one rank */
  MultiSphere* MS;
  int nMS;
  /* ghost send lists (ZJS_VARS.F90:24-27) */
  int npSend[6], npRecv[6], startIdxRecv[6];
  int* partSendIdx[6];
  Parcel* partSend[6];
  int sendCap[6];
  /* cell lists as CSR, per-cell order = insertion order */
  int32_t* cellStart; /* ncell+1 */
  int32_t* cellItems; /* np, 1-based part indices */
  int itemsCap;
  int listsBuilt;
  /* collision lists (ZJS_VARS.F90:30-31) as CSR over locals */
  int32_t* neighPartStart;
  int32_t* neighPartIdx;
  int64_t pairCap;
  /* neighbour cells and delta weights (ZJS_VARS.F90:33-35) for all parcels */
  int32_t* neighCellNo;
  int32_t* neighCellIdx; /* [p*125 + j], 1-based cell ids */
  double* neighCellWeight; /* [(p*125 + j)*3 + comp] */
  int wCap;
  /* fields, Fortran layout with halo */
  double *u, *v, *w, *fx, *fy, *fz, *fxOld, *fyOld, *fzOld, *u0, *v0, *w0;
  /* tangential friction of the marker contacts (orc_set_friction); off while
   * ktRatio == 0.  No counterpart in the reference, whose contact law is normal
   * only (ZJS_COLLISION_DEM.F90:53-57).  History of the last contact-force call:
   * per local of that call its persistent id (the record padding, set by
   * orc_set_parcels) and the range of its contacts, per contact the partner's
   * id (-1: not touching) and the tangential displacement; hMap takes an id to
   * that call's local. */
  double ktRatio, mu;
  int hN;
  int32_t *hGidLocal, *hStart, *hGid, *hMap;
  double* hXi;
  int hMapN;
  char err[256];
};

static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_get_threads(void) { return g_threads; }

static int fail(orc_case* c, int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(c->err, sizeof c->err, fmt, ap);
  va_end(ap);
  return code;
}
const char* orc_last_error(const orc_case* c) { return c ? c->err : "null case"; }

/* ------------------------------------------------------------------ */
/* index maps (ZJS_INIT_DEM.F90:277-296)                               */
static inline int map3Dto1D(const orc_case* c, int i, int j, int k) {
  return (k - c->LG[2]) * c->ni * c->nj + (j - c->LG[1]) * c->ni + (i - c->LG[0]) + 1;
}
static inline void map1Dto3D(const orc_case* c, int idx, int* i, int* j, int* k) {
  int t = idx - 1;
  *i = t % c->ni + c->LG[0];
  t /= c->ni;
  *j = t % c->nj + c->LG[1];
  *k = t / c->nj + c->LG[2];
}
/* field offset of (i,j,k) in the (lg:ug)^3 Fortran-order array */
static inline int64_t fidx(const orc_case* c, int i, int j, int k) {
  return ((int64_t)(k - c->LG[2]) * c->nj + (j - c->LG[1])) * c->ni + (i - c->LG[0]);
}
/* neighCellIdxForCell(j, cell) (ZJS_INIT_DEM.F90:298-331): order kk,jj,ii
 * with ii fastest, -1 outside lg..ug. */
static inline int neighCellIdxForCell(const orc_case* c, int jst, int cell) {
  int i, j, k;
  map1Dto3D(c, cell, &i, &j, &k);
  int kk = jst / 25 - 2, jj = (jst / 5) % 5 - 2, ii = jst % 5 - 2;
  int a = i + ii, b = j + jj, d = k + kk;
  if (a < c->LG[0] || a > c->UG[0] || b < c->LG[1] || b > c->UG[1] || d < c->LG[2] || d > c->UG[2])
    return -1;
  return map3Dto1D(c, a, b, d);
}
/* cell of a position: floor((x-xStart)/di)+SG (ZJS_UPDATE_LIST_DEM.F90:41-43) */
static inline void cellOf(const orc_case* c, const double* x, int* id) {
  id[0] = (int)floor((x[0] - c->start[0]) / c->di) + c->SG[0];
  id[1] = (int)floor((x[1] - c->start[1]) / c->dj) + c->SG[1];
  id[2] = (int)floor((x[2] - c->start[2]) / c->dk) + c->SG[2];
}

/* eta (ZJS_COLLISION_DEM.F90:30): 3.1415926536 is a default-real literal, so
 * its square is formed in single precision and promoted. */
double orc_eta(double e) {
  float pi32 = 3.1415926536f;
  float pi2 = pi32 * pi32;
  return -2 * log(e) / sqrt((double)pi2 + log(e));
}

/* ------------------------------------------------------------------ */
static void* xrealloc(void* p, size_t n) {
  void* q = realloc(p, n ? n : 1);
  return q;
}

orc_case* orc_create(const ibmdem_params* p) {
  if (!p || p->nx < 4 || p->ny < 4 || p->nz < 4) return NULL;
  /* per axis: both faces periodic or both solid walls */
  for (int d = 0; d < 3; ++d)
    if (p->bType[2 * d] != p->bType[2 * d + 1] || (p->bType[2 * d] != 0 && p->bType[2 * d] != 1)) return NULL;
  orc_case* c = (orc_case*)calloc(1, sizeof(orc_case));
  c->p = *p;
  c->n[0] = p->nx;
  c->n[1] = p->ny;
  c->n[2] = p->nz;
  for (int d = 0; d < 3; ++d) {
    c->SG[d] = 1;
    c->EG[d] = c->n[d];
    c->LG[d] = c->SG[d] - HALO;
    c->UG[d] = c->EG[d] + HALO;
  }
  c->ni = c->n[0] + 2 * HALO;
  c->nj = c->n[1] + 2 * HALO;
  c->nk = c->n[2] + 2 * HALO;
  c->ncell = (int64_t)c->ni * c->nj * c->nk;
  /* CopyGridInformationDEM (ZJS_INIT_DEM.F90:333-348) */
  c->di = p->dx;
  c->dj = p->dy;
  c->dk = p->dz;
  c->start[0] = (c->SG[0] - 1) * c->di;
  c->start[1] = (c->SG[1] - 1) * c->dj;
  c->start[2] = (c->SG[2] - 1) * c->dk;
  c->end[0] = (c->EG[0] - 1 + 1) * c->di;
  c->end[1] = (c->EG[1] - 1 + 1) * c->dj;
  c->end[2] = (c->EG[2] - 1 + 1) * c->dk;
  c->len[0] = c->di * c->n[0];
  c->len[1] = c->dj * c->n[1];
  c->len[2] = c->dk * c->n[2];
  /* SetMirrorAndShiftCoords (ZJS_INIT_DEM.F90:258-275) */
  c->coordShift[0] = c->len[0];
  c->coordShift[1] = -c->len[0];
  c->coordShift[2] = c->len[1];
  c->coordShift[3] = -c->len[1];
  c->coordShift[4] = c->len[2];
  c->coordShift[5] = -c->len[2];
  /* walls at the domain's faces: 0 and lGlo on one rank */
  for (int d = 0; d < 3; ++d) {
    c->coordMirror[2 * d] = c->start[d];
    c->coordMirror[2 * d + 1] = c->end[d];
  }
  for (int f = 0; f < 6; ++f)
    for (int d = 0; d < 3; ++d) {
      c->pointBound[f][d] = (f % 2 == 0) ? c->start[d] : c->end[d];
      c->normBound[f][d] = 0.0;
    }
  for (int d = 0; d < 3; ++d) {
    c->normBound[2 * d][d] = 1.0;
    c->normBound[2 * d + 1][d] = -1.0;
  }
  /* InitParameters (ZJS_INIT_DEM.F90:184-195): dtDEM = dt/coupleInterval */
  c->dtDEM = p->dt / p->coupleInterval;
  c->eta = orc_eta(p->ResistCoeff);
  /* Collision (ZJS_COLLISION_DEM.F90:13): (collisionDist*(1+buffer))**2 */
  double cd = p->collisionDist * (1.0 + p->collisionBuffer);
  c->cut2 = cd * cd;
  size_t nf = (size_t)c->ncell;
  double** f[] = {&c->u, &c->v, &c->w, &c->fx, &c->fy, &c->fz, &c->fxOld, &c->fyOld, &c->fzOld, &c->u0, &c->v0, &c->w0};
  for (int q = 0; q < 12; ++q) {
    *f[q] = (double*)calloc(nf, sizeof(double));
    if (!*f[q]) {
      orc_destroy(c);
      return NULL;
    }
  }
  c->cellStart = (int32_t*)calloc(nf + 1, sizeof(int32_t));
  if (!c->cellStart) {
    orc_destroy(c);
    return NULL;
  }
  snprintf(c->err, sizeof c->err, "ok");
  return c;
}

void orc_destroy(orc_case* c) {
  if (!c) return;
  free(c->part);
  free(c->MS);
  for (int f = 0; f < 6; ++f) {
    free(c->partSendIdx[f]);
    free(c->partSend[f]);
  }
  free(c->cellStart);
  free(c->cellItems);
  free(c->neighPartStart);
  free(c->neighPartIdx);
  free(c->neighCellNo);
  free(c->neighCellIdx);
  free(c->neighCellWeight);
  double* f[] = {c->u, c->v, c->w, c->fx, c->fy, c->fz, c->fxOld, c->fyOld, c->fzOld, c->u0, c->v0, c->w0};
  for (int q = 0; q < 12; ++q) free(f[q]);
  free(c->hGidLocal);
  free(c->hStart);
  free(c->hGid);
  free(c->hMap);
  free(c->hXi);
  free(c);
}

/* drop the tangential history: the next contact-force call starts from none */
static void clear_history(orc_case* c) {
  free(c->hGidLocal);
  free(c->hStart);
  free(c->hGid);
  free(c->hMap);
  free(c->hXi);
  c->hGidLocal = c->hStart = c->hGid = c->hMap = NULL;
  c->hXi = NULL;
  c->hN = c->hMapN = 0;
}

int orc_set_friction(orc_case* c, double ktRatio, double mu) {
  if (!(ktRatio >= 0.0) || !(mu >= 0.0)) return fail(c, IBMDEM_EINVAL, "ktRatio and mu must be >= 0");
  c->ktRatio = ktRatio;
  c->mu = mu;
  clear_history(c);
  return 0;
}

static int ensure_parts(orc_case* c, int need) {
  if (need <= c->cap) return 0;
  int nc = c->cap ? c->cap : 1024;
  while (nc < need) nc *= 2;
  Parcel* q = (Parcel*)xrealloc(c->part, (size_t)nc * sizeof(Parcel));
  if (!q) return fail(c, IBMDEM_ENOMEM, "parcel array");
  memset(q + c->cap, 0, (size_t)(nc - c->cap) * sizeof(Parcel));
  c->part = q;
  c->cap = nc;
  return 0;
}
static int push_send(orc_case* c, int f, int i) {
  if (c->npSend[f] + 1 > c->sendCap[f]) {
    int nc = c->sendCap[f] ? 2 * c->sendCap[f] : 1024;
    int* a = (int*)xrealloc(c->partSendIdx[f], (size_t)nc * sizeof(int));
    Parcel* b = (Parcel*)xrealloc(c->partSend[f], (size_t)nc * sizeof(Parcel));
    if (!a || !b) return fail(c, IBMDEM_ENOMEM, "send list");
    c->partSendIdx[f] = a;
    c->partSend[f] = b;
    c->sendCap[f] = nc;
  }
  c->partSend[f][c->npSend[f]] = c->part[i];
  c->partSendIdx[f][c->npSend[f]] = i; /* 0-based here */
  c->npSend[f]++;
  return 0;
}

/* ------------------------------------------------------------------ */
/* state in / out                                                      */
int orc_set_fluid(orc_case* c, const double* u, const double* v, const double* w) {
  size_t nb = (size_t)c->ncell * sizeof(double);
  memcpy(c->u, u, nb);
  memcpy(c->v, v, nb);
  memcpy(c->w, w, nb);
  memcpy(c->u0, u, nb);
  memcpy(c->v0, v, nb);
  memcpy(c->w0, w, nb);
  return 0;
}
int orc_get_fluid(orc_case* c, double* u, double* v, double* w, double* fx, double* fy, double* fz) {
  size_t nb = (size_t)c->ncell * sizeof(double);
  if (u) memcpy(u, c->u, nb);
  if (v) memcpy(v, c->v, nb);
  if (w) memcpy(w, c->w, nb);
  /* interior fx only; halo cells are reported as 0 (deviation 4) */
  double* src[3] = {c->fx, c->fy, c->fz};
  double* dst[3] = {fx, fy, fz};
  for (int q = 0; q < 3; ++q) {
    if (!dst[q]) continue;
    memset(dst[q], 0, nb);
    for (int k = c->SG[2]; k <= c->EG[2]; ++k)
      for (int j = c->SG[1]; j <= c->EG[1]; ++j)
        for (int i = c->SG[0]; i <= c->EG[0]; ++i) dst[q][fidx(c, i, j, k)] = src[q][fidx(c, i, j, k)];
  }
  return 0;
}
int orc_set_parcels(orc_case* c, int32_t np, const ibmdem_parcel* parts) {
  if (np < 0) return fail(c, IBMDEM_EINVAL, "np < 0");
  int rc = ensure_parts(c, np);
  if (rc) return rc;
  memcpy(c->part, parts, (size_t)np * sizeof(Parcel));
  /* the record's padding holds the parcel's persistent id (its index here),
   * which record copies carry to migrated locals and periodic images: the key
   * of the tangential contact history */
  for (int i = 0; i < np; ++i) {
    c->part[i].pType = -1;
    c->part[i].pad_ = i;
  }
  c->np = c->npLocal = np;
  c->listsBuilt = 0;
  clear_history(c);
  return 0;
}
int orc_get_parcels(orc_case* c, ibmdem_parcel* parts, int32_t cap, int32_t* np_out, int32_t* nlocal_out) {
  if (np_out) *np_out = c->np;
  if (nlocal_out) *nlocal_out = c->npLocal;
  if (parts) {
    int n = c->np < cap ? c->np : cap;
    memcpy(parts, c->part, (size_t)n * sizeof(Parcel));
  }
  return 0;
}
int orc_set_bodies(orc_case* c, int32_t n, const ibmdem_multisphere* ms) {
  MultiSphere* q = (MultiSphere*)xrealloc(c->MS, (size_t)(n ? n : 1) * sizeof(MultiSphere));
  if (!q) return fail(c, IBMDEM_ENOMEM, "bodies");
  c->MS = q;
  memcpy(c->MS, ms, (size_t)n * sizeof(MultiSphere));
  c->nMS = n;
  return 0;
}
int orc_get_bodies(orc_case* c, ibmdem_multisphere* ms, int32_t cap, int32_t* n_out) {
  if (n_out) *n_out = c->nMS;
  if (ms) memcpy(ms, c->MS, (size_t)(c->nMS < cap ? c->nMS : cap) * sizeof(MultiSphere));
  return 0;
}
int orc_get_cell_lists(orc_case* c, int32_t* cell_start, int32_t* items, int64_t* ncell_out, int32_t* nitems_out) {
  if (ncell_out) *ncell_out = c->ncell;
  if (nitems_out) *nitems_out = c->np;
  if (!c->listsBuilt) return fail(c, IBMDEM_ESTATE, "lists not built");
  if (cell_start) memcpy(cell_start, c->cellStart, (size_t)(c->ncell + 1) * sizeof(int32_t));
  if (items) memcpy(items, c->cellItems, (size_t)c->np * sizeof(int32_t));
  return 0;
}
int orc_get_collision_lists(orc_case* c, int32_t* start, int32_t* idx, int32_t* nlocal_out, int32_t* npairs_out) {
  if (!c->listsBuilt) return fail(c, IBMDEM_ESTATE, "lists not built");
  if (nlocal_out) *nlocal_out = c->npLocal;
  if (npairs_out) *npairs_out = c->neighPartStart[c->npLocal];
  if (start) memcpy(start, c->neighPartStart, (size_t)(c->npLocal + 1) * sizeof(int32_t));
  if (idx) memcpy(idx, c->neighPartIdx, (size_t)c->neighPartStart[c->npLocal] * sizeof(int32_t));
  return 0;
}
int orc_get_weights(orc_case* c, int32_t n, double* w, int32_t* cells) {
  if (n > c->np || n > c->wCap) return fail(c, IBMDEM_EINVAL, "weights for %d parcels not available", n);
  for (int p = 0; p < n; ++p) {
    int cnt = c->neighCellNo[p];
    for (int j = 0; j < NST; ++j) {
      if (cells) cells[p * NST + j] = j < cnt ? c->neighCellIdx[p * NST + j] : 0;
      for (int q = 0; q < 3; ++q)
        if (w) w[((size_t)p * NST + j) * 3 + q] = j < cnt ? c->neighCellWeight[((size_t)p * NST + j) * 3 + q] : 0.0;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* cell lists (ZJS_UPDATE_LIST_DEM.F90:2-177)                          */

/* CompressDEM (ZJS_UPDATE_LIST_DEM.F90:2-27) */
static void CompressDEM(orc_case* c) {
  int np_updated = 0;
  for (int i = 0; i < c->np; ++i) {
    if (c->part[i].pType == -1) {
      int id[3];
      cellOf(c, c->part[i].x, id);
      if (id[0] >= c->SG[0] && id[0] <= c->EG[0] && id[1] >= c->SG[1] && id[1] <= c->EG[1] && id[2] >= c->SG[2] &&
          id[2] <= c->EG[2]) {
        c->part[np_updated] = c->part[i];
        c->part[np_updated].pType = -1;
        np_updated++;
      }
    }
  }
  c->np = np_updated;
  c->npLocal = c->np;
}

/* PutParcelsIntoCellsDEM (ZJS_UPDATE_LIST_DEM.F90:29-97); the partIdxInCell
 * append is deferred to build_cell_csr(), which inserts in part order. */
static int PutParcelsIntoCellsDEM(orc_case* c, int npStart, int npEnd, int mode) {
  for (int i = npStart; i < npEnd; ++i) {
    int id[3];
    cellOf(c, c->part[i].x, id);
    if (id[0] < c->LG[0] || id[0] > c->UG[0] || id[1] < c->LG[1] || id[1] > c->UG[1] || id[2] < c->LG[2] ||
        id[2] > c->UG[2])
      return fail(c, IBMDEM_ERANGE, "parcel %d at (%g,%g,%g) exceeds the region", i + 1, c->part[i].x[0],
                  c->part[i].x[1], c->part[i].x[2]);
    c->part[i].localIdx = i + 1;
    c->part[i].cellIdx = map3Dto1D(c, id[0], id[1], id[2]);
    if (mode == 0) c->part[i].pType = -1;
    int rc = 0;
    if (mode <= 0) {
      if (id[0] <= c->SG[0] + HALO - 1 && id[0] >= c->SG[0]) rc |= push_send(c, 0, i);
      if (id[0] >= c->EG[0] - HALO + 1 && id[0] <= c->EG[0]) rc |= push_send(c, 1, i);
    }
    if (mode <= 1) {
      if (id[1] <= c->SG[1] + HALO - 1 && id[1] >= c->SG[1]) rc |= push_send(c, 2, i);
      if (id[1] >= c->EG[1] - HALO + 1 && id[1] <= c->EG[1]) rc |= push_send(c, 3, i);
    }
    if (mode <= 2) {
      if (id[2] <= c->SG[2] + HALO - 1 && id[2] >= c->SG[2]) rc |= push_send(c, 4, i);
      if (id[2] >= c->EG[2] - HALO + 1 && id[2] <= c->EG[2]) rc |= push_send(c, 5, i);
    }
    if (rc) return IBMDEM_ENOMEM;
  }
  return 0;
}

/* RebuildParcelInCellListForGhostRegionDEM (ZJS_UPDATE_LIST_DEM.F90:122-177)
 * with MyMPISendAndRecv (ZJS_MPI_DEM.F90:2-100) to this rank itself. */
static int RebuildParcelInCellListForGhostRegionDEM(orc_case* c) {
  for (int idx = 0; idx < 6; ++idx) {
    int idxSend = idx;
    int idxRecv = (idx % 2 == 0) ? idx + 1 : idx - 1;
    int nSend = c->npSend[idx];
    int dim = idx / 2;
    if (c->p.bType[idxRecv] == 1) {
      /* no rank beyond the wall (neighCpu = -1): UpdateFullInfoForSolidOutletBoundary
       * (ZJS_MPI_DEM.F90:173-210) mirrors the parcels near face idxRecv itself */
      int nRecv = c->npSend[idxRecv];
      c->npRecv[idxRecv] = nRecv;
      int rc = ensure_parts(c, c->np + nRecv);
      if (rc) return rc;
      for (int i = 0; i < nRecv; ++i) {
        Parcel* d = &c->part[c->np + i];
        *d = c->part[c->partSendIdx[idxRecv][i]];
        d->x[dim] = 2 * c->coordMirror[idxRecv] - d->x[dim];
        d->v[dim] = -d->v[dim];
        d->pType = 1;
      }
      rc = PutParcelsIntoCellsDEM(c, c->np, c->np + nRecv, dim + 1);
      if (rc) return rc;
      c->startIdxRecv[idxRecv] = c->np;
      c->np += nRecv;
      continue;
    }
    /* periodic: shift the copies (ZJS_UPDATE_LIST_DEM.F90:147-151) */
    for (int i = 0; i < nSend; ++i) c->partSend[idxSend][i].x[dim] = c->partSend[idxSend][i].x[dim] + c->coordShift[idxSend];
    /* receive into part(np+1 : np+nRecv): fields of ZJS_MPI_DEM.F90:82-95 */
    int nRecv = nSend;
    c->npRecv[idxRecv] = nRecv;
    int rc = ensure_parts(c, c->np + nRecv);
    if (rc) return rc;
    for (int i = 0; i < nRecv; ++i) {
      Parcel* d = &c->part[c->np + i];
      const Parcel* s = &c->partSend[idxSend][i];
      d->globalIdx = s->globalIdx;
      d->localIdx = s->localIdx;
      d->cellIdx = s->cellIdx;
      d->pType = s->pType;
      d->MSIdx = s->MSIdx;
      d->radeff = s->radeff;
      d->rad = s->rad;
      d->rho = s->rho;
      d->vol = s->vol;
      d->m = s->m;
      memcpy(d->x, s->x, sizeof d->x);
      memcpy(d->v, s->v, sizeof d->v);
      memcpy(d->fcol, s->fcol, sizeof d->fcol);
      memcpy(d->fdrag, s->fdrag, sizeof d->fdrag);
      /* not sent (ZJS_MPI_DEM.F90:82-95): the reference leaves the slot's old
       * contents there; they are defined as zero here (deviation 5) */
      memset(d->vgap, 0, sizeof d->vgap);
      d->wdrag = 0.0;
    }
    rc = PutParcelsIntoCellsDEM(c, c->np, c->np + nRecv, dim + 1);
    if (rc) return rc;
    c->startIdxRecv[idxRecv] = c->np; /* 0-based */
    c->np += nRecv;
  }
  return 0;
}

static int build_cell_csr(orc_case* c) {
  if (c->itemsCap < c->np) {
    int32_t* q = (int32_t*)xrealloc(c->cellItems, (size_t)c->np * sizeof(int32_t));
    if (!q) return fail(c, IBMDEM_ENOMEM, "cell items");
    c->cellItems = q;
    c->itemsCap = c->np;
  }
  /* npPartInCell (ZJS_UPDATE_LIST_DEM.F90:50) as counts, then offsets:
   * cellStart[cell-1] = first item of cell, cellStart[cell] = one past it. */
  memset(c->cellStart, 0, (size_t)(c->ncell + 1) * sizeof(int32_t));
  for (int i = 0; i < c->np; ++i) c->cellStart[c->part[i].cellIdx]++;
  for (int64_t q = 0; q < c->ncell; ++q) c->cellStart[q + 1] += c->cellStart[q];
  int32_t* cursor = (int32_t*)malloc((size_t)c->ncell * sizeof(int32_t));
  if (!cursor) return fail(c, IBMDEM_ENOMEM, "cursor");
  memcpy(cursor, c->cellStart, (size_t)c->ncell * sizeof(int32_t));
  /* partIdxInCell (ZJS_UPDATE_LIST_DEM.F90:51): append in part order */
  for (int i = 0; i < c->np; ++i) c->cellItems[cursor[c->part[i].cellIdx - 1]++] = i + 1;
  free(cursor);
  return 0;
}

/* RebuildParcelInCellListDEM (ZJS_UPDATE_LIST_DEM.F90:99-120) */
static int RebuildParcelInCellListDEM(orc_case* c) {
  CompressDEM(c);
  for (int f = 0; f < 6; ++f) c->npSend[f] = c->npRecv[f] = 0;
  int rc = PutParcelsIntoCellsDEM(c, 0, c->np, 0);
  if (rc) return rc;
  rc = RebuildParcelInCellListForGhostRegionDEM(c);
  if (rc) return rc;
  return build_cell_csr(c);
}

/* Collision (ZJS_COLLISION_DEM.F90:2-19) */
static inline int Collision(const orc_case* c, const Parcel* a, const Parcel* b) {
  double xij1 = a->x[0] - b->x[0];
  double xij2 = a->x[1] - b->x[1];
  double xij3 = a->x[2] - b->x[2];
  double distSqr = xij1 * xij1 + xij2 * xij2 + xij3 * xij3;
  return distSqr < c->cut2;
}

/* RebuildParcelCollisionListDEM (ZJS_UPDATE_LIST_DEM.F90:248-286) */
static int scan_pairs(orc_case* c, int ii, int32_t* out) {
  int cnt = 0;
  const Parcel* pi = &c->part[ii];
  for (int j = 0; j < NST; ++j) {
    int cellIdxTmp = neighCellIdxForCell(c, j, pi->cellIdx);
    if (cellIdxTmp == -1) continue;
    int32_t s = c->cellStart[cellIdxTmp - 1], e = c->cellStart[cellIdxTmp];
    for (int k = s; k < e; ++k) {
      int jj = c->cellItems[k] - 1;
      const Parcel* pj = &c->part[jj];
      if (pi->MSIdx != pj->MSIdx) {
        if (Collision(c, pi, pj) && pj->pType == -1 && ii != jj) {
          if (out) out[cnt] = jj + 1;
          cnt++;
        }
      }
    }
  }
  return cnt;
}
static int RebuildParcelCollisionListDEM(orc_case* c) {
  int n = c->npLocal;
  int32_t* st = (int32_t*)xrealloc(c->neighPartStart, (size_t)(n + 1) * sizeof(int32_t));
  if (!st) return fail(c, IBMDEM_ENOMEM, "pair starts");
  c->neighPartStart = st;
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads)
  for (int i = 0; i < n; ++i) st[i + 1] = scan_pairs(c, i, NULL);
  st[0] = 0;
  for (int i = 0; i < n; ++i) st[i + 1] += st[i];
  if (st[n] > c->pairCap) {
    int32_t* q = (int32_t*)xrealloc(c->neighPartIdx, (size_t)st[n] * sizeof(int32_t));
    if (!q) return fail(c, IBMDEM_ENOMEM, "pairs");
    c->neighPartIdx = q;
    c->pairCap = st[n];
  }
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads)
  for (int i = 0; i < n; ++i) scan_pairs(c, i, c->neighPartIdx + st[i]);
  return 0;
}

/* RebuildNeighborCellListForParcelsDEM (ZJS_UPDATE_LIST_DEM.F90:288-321) */
static int RebuildNeighborCellListForParcelsDEM(orc_case* c) {
  if (c->wCap < c->np) {
    int nc = c->np + c->np / 8 + 64;
    int32_t* a = (int32_t*)xrealloc(c->neighCellNo, (size_t)nc * sizeof(int32_t));
    int32_t* b = (int32_t*)xrealloc(c->neighCellIdx, (size_t)nc * NST * sizeof(int32_t));
    double* w = (double*)xrealloc(c->neighCellWeight, (size_t)nc * NST * 3 * sizeof(double));
    if (!a || !b || !w) return fail(c, IBMDEM_ENOMEM, "neighbour cell lists");
    c->neighCellNo = a;
    c->neighCellIdx = b;
    c->neighCellWeight = w;
    c->wCap = nc;
  }
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int i = 0; i < c->np; ++i) {
    int cnt = 0;
    for (int j = 0; j < NST; ++j) {
      int t = neighCellIdxForCell(c, j, c->part[i].cellIdx);
      if (t != -1) c->neighCellIdx[(size_t)i * NST + cnt++] = t;
    }
    c->neighCellNo[i] = cnt;
  }
  return 0;
}

/* RebuildAllListOrNot (ZJS_EVOLUTION_DEM.F90:34-41) */
int orc_RebuildAllListOrNot(orc_case* c) {
  int rc = RebuildParcelInCellListDEM(c);
  if (rc) return rc;
  rc = RebuildParcelCollisionListDEM(c);
  if (rc) return rc;
  rc = RebuildNeighborCellListForParcelsDEM(c);
  if (rc) return rc;
  c->listsBuilt = 1;
  return 0;
}

/* ------------------------------------------------------------------ */
/* delta function and weights                                          */

/* one axis of DeltaFunction3D (interpolation.F90:7-30) */
static inline double delta1(double xcp, double h) {
  double r = fabs(xcp / h);
  double w;
  if (r <= 0.5)
    w = (1 + sqrt(1 - 3 * r * r)) / 3;
  else if (r <= 1.5)
    w = (5 - 3 * r - sqrt(1 - 3 * ((1 - r) * (1 - r)))) / 6;
  else
    w = 0;
  return w;
}
/* DeltaFunction3D (interpolation.F90:2-33) */
static inline double DeltaFunction3D(const orc_case* c, double a, double b, double d) {
  double w1 = delta1(a, c->p.dx), w2 = delta1(b, c->p.dy), w3 = delta1(d, c->p.dz);
  return w1 * w2 * w3 / (c->p.dx * c->p.dy * c->p.dz);
}
/* GetWeight (ZJS_INTERPOLATE_DEM.F90:2-17) */
static inline void GetWeight(const orc_case* c, const double* xp, const double* xcell, double* weight) {
  double deltax1 = xp[0] - xcell[0];
  double deltax2 = xp[1] - xcell[1];
  double deltax3 = xp[2] - xcell[2];
  weight[0] = DeltaFunction3D(c, deltax1 + 0.5 * c->di, deltax2, deltax3);
  weight[1] = DeltaFunction3D(c, deltax1, deltax2 + 0.5 * c->dj, deltax3);
  weight[2] = DeltaFunction3D(c, deltax1, deltax2, deltax3 + 0.5 * c->dk);
}
static void weights_range(orc_case* c, int p0, int p1) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int i = p0; i < p1; ++i) {
    const double* xp = c->part[i].x;
    int cnt = c->neighCellNo[i];
    for (int j = 0; j < cnt; ++j) {
      int a, b, d;
      map1Dto3D(c, c->neighCellIdx[(size_t)i * NST + j], &a, &b, &d);
      /* xc = (i-0.5)dx (initialization.F90:251-253) */
      double xcell[3] = {(a - 0.5) * c->p.dx, (b - 0.5) * c->p.dy, (d - 0.5) * c->p.dz};
      GetWeight(c, xp, xcell, &c->neighCellWeight[((size_t)i * NST + j) * 3]);
    }
  }
}
/* UpdateLocalCellWeightListDEM (ZJS_UPDATE_LIST_DEM.F90:323-370) */
int orc_UpdateLocalCellWeightListDEM(orc_case* c) {
  if (!c->listsBuilt) return fail(c, IBMDEM_ESTATE, "lists not built");
  weights_range(c, 0, c->npLocal);
  return 0;
}
/* UpdateGhostCellWeightListDEM (ZJS_UPDATE_LIST_DEM.F90:372-416) */
int orc_UpdateGhostCellWeightListDEM(orc_case* c) {
  if (!c->listsBuilt) return fail(c, IBMDEM_ESTATE, "lists not built");
  weights_range(c, c->npLocal, c->np);
  return 0;
}

/* UpdateParcelInfoInGhostRegion (ZJS_UPDATE_LIST_DEM.F90:179-246) with
 * MyMPIUpdateVelocityAndPosition (ZJS_MPI_DEM.F90:102-171) to this rank. */
int orc_UpdateParcelInfoInGhostRegion(orc_case* c) {
  for (int idx = 0; idx < 6; ++idx) {
    int idxSend = idx;
    int idxRecv = (idx % 2 == 0) ? idx + 1 : idx - 1;
    int nSend = c->npSend[idx];
    int dim = idx / 2;
    for (int i = 0; i < nSend; ++i) {
      Parcel* s = &c->partSend[idx][i];
      const Parcel* o = &c->part[c->partSendIdx[idx][i]];
      s->MSIdx = o->MSIdx;
      memcpy(s->x, o->x, sizeof s->x);
      memcpy(s->v, o->v, sizeof s->v);
      s->wsum = o->wsum;
      memcpy(s->fdrag, o->fdrag, sizeof s->fdrag);
    }
    if (c->p.bType[idxRecv] == 1) {
      /* UpdatePartInfoForSolidOutletBoundary (ZJS_MPI_DEM.F90:222-269) */
      int nRecv = c->npSend[idxRecv];
      for (int i = 0; i < nRecv; ++i) {
        Parcel* d = &c->part[c->startIdxRecv[idxRecv] + i];
        const Parcel* o = &c->part[c->partSendIdx[idxRecv][i]];
        memcpy(d->x, o->x, sizeof d->x);
        memcpy(d->v, o->v, sizeof d->v);
        memcpy(d->fdrag, o->fdrag, sizeof d->fdrag);
        d->wsum = o->wsum;
        d->x[dim] = 2 * c->coordMirror[idxRecv] - d->x[dim];
        d->v[dim] = -d->v[dim];
        d->pType = 1;
      }
      continue;
    }
    for (int i = 0; i < nSend; ++i) c->partSend[idxSend][i].x[dim] = c->partSend[idxSend][i].x[dim] + c->coordShift[idxSend];
    int nRecv = c->npRecv[idxRecv];
    for (int i = 0; i < nRecv; ++i) {
      Parcel* d = &c->part[c->startIdxRecv[idxRecv] + i];
      const Parcel* s = &c->partSend[idxSend][i];
      d->MSIdx = s->MSIdx;
      memcpy(d->x, s->x, sizeof d->x);
      memcpy(d->v, s->v, sizeof d->v);
      d->wsum = s->wsum;
      memcpy(d->fdrag, s->fdrag, sizeof d->fdrag);
    }
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* contacts                                                            */

/* CalculateCollisionForce with tangential friction (orc_set_friction; not in
 * the reference).  The normal part is the reference's law below, term by term.
 * For a touching pair (deltan > 0) with relative marker velocity
 * u = v_i - v_j (marker velocities include their body's rotation):
 *   vt = u - vn n (vn as the normal law forms it);
 *   h  = the pair's tangential displacement of the last call (keyed by the
 *        persistent ids of both parcels, 0 when new), projected on the tangent
 *        plane, h - (n.h) n, then h + dtDEM vt;
 *   kt = ktRatio kn, etat = eta sqrt(meff kt), ft = -kt h - etat vt;
 *   Coulomb: when |ft| > mu |fn| (fn = kn deltan - etan vn), ft is scaled to
 *        mu |fn| and h reset to the sliding value -(ft + etat vt) / kt;
 *   fcol_i += n fn + ft, component by component.
 * A listed pair that does not touch keeps no history. */
static int collision_force_friction(orc_case* c) {
  const double eta = c->eta, knCoeff = c->p.knCoeff, di = c->di, dtDEM = c->dtDEM;
  const double ktRatio = c->ktRatio, mu = c->mu;
  const int nl = c->npLocal;
  const int64_t npairs = c->neighPartStart[nl];
  int32_t* nGid = (int32_t*)malloc((size_t)(npairs ? npairs : 1) * sizeof(int32_t));
  double* nXi = (double*)malloc((size_t)(npairs ? npairs : 1) * 3 * sizeof(double));
  int32_t* nStart = (int32_t*)malloc((size_t)(nl + 1) * sizeof(int32_t));
  int32_t* nGidLocal = (int32_t*)malloc((size_t)(nl ? nl : 1) * sizeof(int32_t));
  if (!nGid || !nXi || !nStart || !nGidLocal) {
    free(nGid);
    free(nXi);
    free(nStart);
    free(nGidLocal);
    return fail(c, IBMDEM_ENOMEM, "tangential history");
  }
  memcpy(nStart, c->neighPartStart, (size_t)(nl + 1) * sizeof(int32_t));
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads)
  for (int ii = 0; ii < nl; ++ii) {
    Parcel* pi = &c->part[ii];
    const int gi = pi->pad_;
    nGidLocal[ii] = gi;
    const int o = (gi >= 0 && gi < c->hMapN) ? c->hMap[gi] : -1;
    const int os = o >= 0 ? c->hStart[o] : 0, oe = o >= 0 ? c->hStart[o + 1] : 0;
    pi->fcol[0] = 0;
    pi->fcol[1] = 0;
    pi->fcol[2] = 0;
    for (int q = c->neighPartStart[ii]; q < c->neighPartStart[ii + 1]; ++q) {
      const Parcel* pj = &c->part[c->neighPartIdx[q] - 1];
      double r1 = pi->x[0] - pj->x[0];
      double r2 = pi->x[1] - pj->x[1];
      double r3 = pi->x[2] - pj->x[2];
      double dist = sqrt(r1 * r1 + r2 * r2 + r3 * r3);
      double n1 = r1 / dist, n2 = r2 / dist, n3 = r3 / dist;
      double meff = 2 * pi->m * pj->m / (pi->m + pj->m);
      double rij = pi->radeff + pj->radeff;
      double deltan = rij - dist;
      double kn = knCoeff / (0.1 * di) * meff;
      double etan = eta * sqrt(meff * kn);
      double f1 = 0, f2 = 0, f3 = 0;
      double u1 = pi->v[0] - pj->v[0], u2 = pi->v[1] - pj->v[1], u3 = pi->v[2] - pj->v[2];
      double vnij = n1 * u1 + n2 * u2 + n3 * u3;
      double h1 = 0, h2 = 0, h3 = 0;
      int hg = -1;
      if (deltan > 0) {
        double fn = kn * deltan - etan * vnij;
        double vt1 = u1 - vnij * n1, vt2 = u2 - vnij * n2, vt3 = u3 - vnij * n3;
        for (int t = os; t < oe; ++t)
          if (c->hGid[t] == pj->pad_) {
            h1 = c->hXi[3 * (size_t)t];
            h2 = c->hXi[3 * (size_t)t + 1];
            h3 = c->hXi[3 * (size_t)t + 2];
            break;
          }
        double hn = n1 * h1 + n2 * h2 + n3 * h3;
        h1 = h1 - hn * n1;
        h2 = h2 - hn * n2;
        h3 = h3 - hn * n3;
        h1 = h1 + dtDEM * vt1;
        h2 = h2 + dtDEM * vt2;
        h3 = h3 + dtDEM * vt3;
        double kt = ktRatio * kn;
        double etat = eta * sqrt(meff * kt);
        double ft1 = -kt * h1 - etat * vt1, ft2 = -kt * h2 - etat * vt2, ft3 = -kt * h3 - etat * vt3;
        double ftm = sqrt(ft1 * ft1 + ft2 * ft2 + ft3 * ft3);
        double lim = mu * fabs(fn);
        if (ftm > lim) {
          double sc = lim / ftm;
          ft1 = ft1 * sc;
          ft2 = ft2 * sc;
          ft3 = ft3 * sc;
          h1 = -(ft1 + etat * vt1) / kt;
          h2 = -(ft2 + etat * vt2) / kt;
          h3 = -(ft3 + etat * vt3) / kt;
        }
        f1 = n1 * fn + ft1;
        f2 = n2 * fn + ft2;
        f3 = n3 * fn + ft3;
        hg = pj->pad_;
      }
      nGid[q] = hg;
      nXi[3 * (size_t)q] = h1;
      nXi[3 * (size_t)q + 1] = h2;
      nXi[3 * (size_t)q + 2] = h3;
      pi->fcol[0] = pi->fcol[0] + f1;
      pi->fcol[1] = pi->fcol[1] + f2;
      pi->fcol[2] = pi->fcol[2] + f3;
    }
  }
  int maxg = -1;
  for (int ii = 0; ii < nl; ++ii) maxg = nGidLocal[ii] > maxg ? nGidLocal[ii] : maxg;
  int32_t* map = (int32_t*)malloc((size_t)(maxg + 2) * sizeof(int32_t));
  if (!map) {
    free(nGid);
    free(nXi);
    free(nStart);
    free(nGidLocal);
    return fail(c, IBMDEM_ENOMEM, "tangential history");
  }
  for (int g = 0; g <= maxg + 1; ++g) map[g] = -1;
  for (int ii = 0; ii < nl; ++ii)
    if (nGidLocal[ii] >= 0) map[nGidLocal[ii]] = ii;
  clear_history(c);
  c->hN = nl;
  c->hGidLocal = nGidLocal;
  c->hStart = nStart;
  c->hGid = nGid;
  c->hXi = nXi;
  c->hMap = map;
  c->hMapN = maxg + 2;
  return 0;
}

/* the tangential history of the last contact-force call as CSR over that
 * call's locals: start[nl+1], partner id (-1: not touching) and 3
 * displacement components per contact; pass NULL to query the sizes */
int orc_get_friction_history(orc_case* c, int32_t* start, int32_t* gid, double* xi, int32_t* nl_out,
                             int32_t* n_out) {
  if (nl_out) *nl_out = c->hN;
  if (n_out) *n_out = c->hN ? c->hStart[c->hN] : 0;
  if (!c->hN) return 0;
  if (start) memcpy(start, c->hStart, (size_t)(c->hN + 1) * sizeof(int32_t));
  if (gid) memcpy(gid, c->hGid, (size_t)c->hStart[c->hN] * sizeof(int32_t));
  if (xi) memcpy(xi, c->hXi, (size_t)c->hStart[c->hN] * 3 * sizeof(double));
  return 0;
}

/* CalculateCollisionForce (ZJS_COLLISION_DEM.F90:21-74) */
int orc_CalculateCollisionForce(orc_case* c) {
  if (!c->listsBuilt) return fail(c, IBMDEM_ESTATE, "lists not built");
  if (c->ktRatio > 0.0) return collision_force_friction(c);
  const double eta = c->eta;
  const double knCoeff = c->p.knCoeff, di = c->di;
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads)
  for (int ii = 0; ii < c->npLocal; ++ii) {
    Parcel* pi = &c->part[ii];
    pi->fcol[0] = 0;
    pi->fcol[1] = 0;
    pi->fcol[2] = 0;
    for (int q = c->neighPartStart[ii]; q < c->neighPartStart[ii + 1]; ++q) {
      const Parcel* pj = &c->part[c->neighPartIdx[q] - 1];
      double r1 = pi->x[0] - pj->x[0];
      double r2 = pi->x[1] - pj->x[1];
      double r3 = pi->x[2] - pj->x[2];
      double dist = sqrt(r1 * r1 + r2 * r2 + r3 * r3);
      double n1 = r1 / dist, n2 = r2 / dist, n3 = r3 / dist;
      double meff = 2 * pi->m * pj->m / (pi->m + pj->m);
      double rij = pi->radeff + pj->radeff;
      double deltan = rij - dist;
      double kn = knCoeff / (0.1 * di) * meff;
      double etan = eta * sqrt(meff * kn);
      double f1 = 0, f2 = 0, f3 = 0;
      double vnij = n1 * (pi->v[0] - pj->v[0]) + n2 * (pi->v[1] - pj->v[1]) + n3 * (pi->v[2] - pj->v[2]);
      if (deltan > 0) {
        f1 = n1 * (kn * deltan - etan * vnij);
        f2 = n2 * (kn * deltan - etan * vnij);
        f3 = n3 * (kn * deltan - etan * vnij);
      }
      pi->fcol[0] = pi->fcol[0] + f1;
      pi->fcol[1] = pi->fcol[1] + f2;
      pi->fcol[2] = pi->fcol[2] + f3;
    }
  }
  return 0;
}

/* WallProbeCollision (ZJS_COLLISION_DEM.F90:150-179): the contact point is
 * inside the quadrilateral when the angles it sees the four edges under sum
 * to 2 pi (within 0.001 pi); a NaN angle sum counts as inside, as the
 * reference's comparison is false for it. */
static int WallProbeCollision(double cp1, double cp2, double cp3, const ibmdem_wall_probe* prob) {
  double theta = 0.0;
  for (int i = 0; i < 4; ++i) {
    int idxi = i, idxj = i + 1;
    if (idxj > 3) idxj = idxj - 4;
    double ni1 = prob->points[idxi][0] - cp1;
    double ni2 = prob->points[idxi][1] - cp2;
    double ni3 = prob->points[idxi][2] - cp3;
    double nj1 = prob->points[idxj][0] - cp1;
    double nj2 = prob->points[idxj][1] - cp2;
    double nj3 = prob->points[idxj][2] - cp3;
    double thetai = (ni1 * nj1 + ni2 * nj2 + ni3 * nj3) /
                    (sqrt(ni1 * ni1 + ni2 * ni2 + ni3 * ni3) * sqrt(nj1 * nj1 + nj2 * nj2 + nj3 * nj3));
    thetai = acos(thetai);
    theta = theta + thetai;
  }
  double pi = acos(-1.0);
  return fabs(theta - 2 * pi) > 0.001 * pi ? 0 : 1;
}

/* CalculateSolidBoundaryCollisionForce (ZJS_COLLISION_DEM.F90:76-148): the
 * parcel-plane spring-dashpot for local parcels in the first or last interior
 * cell layer, face by face, added to fcol after the pair forces; the normal
 * spring part is summed into every probe of the face that contains the contact
 * point, in part order.  The per-hit log line the reference appends to its
 * log file is not written. */
int orc_CalculateSolidBoundaryCollisionForce(orc_case* c) {
  if (!c->listsBuilt) return fail(c, IBMDEM_ESTATE, "lists not built");
  for (int q = 0; q < c->nProbe; ++q) memset(c->probe[q].force, 0, sizeof c->probe[q].force);
  const double eta = c->eta;
  const double knCoeff = c->p.knCoeff, di = c->di;
  for (int i = 0; i < c->npLocal; ++i) {
    Parcel* pi = &c->part[i];
    int cellIdx1, cellIdx2, cellIdx3;
    map1Dto3D(c, pi->cellIdx, &cellIdx1, &cellIdx2, &cellIdx3);
    double xij1 = pi->x[0], xij2 = pi->x[1], xij3 = pi->x[2];
    if (!(cellIdx1 == c->SG[0] || cellIdx1 == c->EG[0] || cellIdx2 == c->SG[1] || cellIdx2 == c->EG[1] ||
          cellIdx3 == c->SG[2] || cellIdx3 == c->EG[2]))
      continue;
    for (int j = 0; j < 6; ++j) {
      if (c->p.bType[j] != 1) continue;
      double p1 = c->pointBound[j][0], p2 = c->pointBound[j][1], p3 = c->pointBound[j][2];
      double n1 = c->normBound[j][0], n2 = c->normBound[j][1], n3 = c->normBound[j][2];
      double r1 = xij1 - p1, r2 = xij2 - p2, r3 = xij3 - p3;
      double dist = r1 * n1 + r2 * n2 + r3 * n3;
      double cp1 = xij1 - dist * n1;
      double cp2 = xij2 - dist * n2;
      double cp3 = xij3 - dist * n3;
      double meff = pi->m;
      double rij = pi->radeff;
      double deltan = rij - dist;
      double kn = knCoeff / (0.1 * di) * meff;
      double etan = eta * sqrt(meff * kn);
      double vnij = n1 * pi->v[0] + n2 * pi->v[1] + n3 * pi->v[2];
      if (deltan > 0) {
        double f1 = n1 * (kn * deltan - etan * vnij);
        double f2 = n2 * (kn * deltan - etan * vnij);
        double f3 = n3 * (kn * deltan - etan * vnij);
        double fn1 = n1 * kn * deltan;
        double fn2 = n2 * kn * deltan;
        double fn3 = n3 * kn * deltan;
        pi->fcol[0] = pi->fcol[0] + f1;
        pi->fcol[1] = pi->fcol[1] + f2;
        pi->fcol[2] = pi->fcol[2] + f3;
        for (int k = 0; k < c->nProbe; ++k) {
          ibmdem_wall_probe* pr = &c->probe[k];
          if (pr->face != j + 1) continue;
          if (WallProbeCollision(cp1, cp2, cp3, pr)) {
            pr->force[0] = pr->force[0] + fn1;
            pr->force[1] = pr->force[1] + fn2;
            pr->force[2] = pr->force[2] + fn3;
          }
        }
      }
    }
  }
  return 0;
}

int orc_set_wall_probes(orc_case* c, int32_t n, const ibmdem_wall_probe* probes) {
  if (n < 0 || n > IBMDEM_MAX_WALL_PROBES || (n > 0 && !probes)) return fail(c, IBMDEM_EINVAL, "probe count");
  for (int q = 0; q < n; ++q)
    if (probes[q].face < 1 || probes[q].face > 6 || c->p.bType[probes[q].face - 1] != 1)
      return fail(c, IBMDEM_EINVAL, "probe %d is not on a wall face", q);
  memcpy(c->probe, probes, (size_t)n * sizeof *probes);
  for (int q = 0; q < n; ++q) memset(c->probe[q].force, 0, sizeof c->probe[q].force);
  c->nProbe = n;
  return 0;
}

int orc_get_wall_probes(orc_case* c, ibmdem_wall_probe* probes, int32_t cap, int32_t* n_out) {
  if (n_out) *n_out = c->nProbe;
  if (probes) memcpy(probes, c->probe, (size_t)(cap < c->nProbe ? cap : c->nProbe) * sizeof *probes);
  return 0;
}

/* ------------------------------------------------------------------ */
/* immersed boundary                                                   */

/* UpdateFluidVelocityOnLagrangianPoints (ZJS_VOLUMEFRACTION_DEM.F90:2-36) */
int orc_UpdateFluidVelocityOnLagrangianPoints(orc_case* c) {
  if (!c->listsBuilt) return fail(c, IBMDEM_ESTATE, "lists not built");
  const double relaxfactor = 1.0;
  const double dx = c->p.dx, dy = c->p.dy, dz = c->p.dz, dt = c->p.dt;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int i = 0; i < c->npLocal; ++i) {
    Parcel* p = &c->part[i];
    double ulp = 0, vlp = 0, wlp = 0;
    for (int j = 0; j < c->neighCellNo[i]; ++j) {
      int a, b, d;
      map1Dto3D(c, c->neighCellIdx[(size_t)i * NST + j], &a, &b, &d);
      const double* wt = &c->neighCellWeight[((size_t)i * NST + j) * 3];
      int64_t f = fidx(c, a, b, d);
      ulp = ulp + wt[0] * c->u[f] * dx * dy * dz;
      vlp = vlp + wt[1] * c->v[f] * dx * dy * dz;
      wlp = wlp + wt[2] * c->w[f] * dx * dy * dz;
    }
    p->vgap[0] = ulp - p->v[0];
    p->vgap[1] = vlp - p->v[1];
    p->vgap[2] = wlp - p->v[2];
    p->fdrag[0] = p->fdrag[0] + relaxfactor * (ulp - p->v[0]) / dt;
    p->fdrag[1] = p->fdrag[1] + relaxfactor * (vlp - p->v[1]) / dt;
    p->fdrag[2] = p->fdrag[2] + relaxfactor * (wlp - p->v[2]) / dt;
  }
  return 0;
}

/* UpdateMomentumSourceTerm (ZJS_VOLUMEFRACTION_DEM.F90:38-67).  Threads own
 * disjoint z-slabs of cells and each visits the parcels in part order, so every
 * cell accumulates its contributions in the reference's order. */
int orc_UpdateMomentumSourceTerm(orc_case* c) {
  if (!c->listsBuilt) return fail(c, IBMDEM_ESTATE, "lists not built");
  size_t nb = (size_t)c->ncell * sizeof(double);
  memcpy(c->fxOld, c->fx, nb);
  memcpy(c->fyOld, c->fy, nb);
  memcpy(c->fzOld, c->fz, nb);
  memset(c->fx, 0, nb);
  memset(c->fy, 0, nb);
  memset(c->fz, 0, nb);
  int nth = g_threads;
  int kz0 = c->LG[2], kz1 = c->UG[2] + 1;
#pragma omp parallel num_threads(nth)
  {
    int t = 0, T = 1;
#ifdef _OPENMP
    t = omp_get_thread_num();
    T = omp_get_num_threads();
#endif
    int span = kz1 - kz0;
    int lo = kz0 + (int)((int64_t)span * t / T), hi = kz0 + (int)((int64_t)span * (t + 1) / T);
    for (int i = 0; i < c->np; ++i) {
      const Parcel* p = &c->part[i];
      int a, b, d;
      map1Dto3D(c, p->cellIdx, &a, &b, &d);
      if (d + 2 < lo || d - 2 >= hi) continue;
      for (int j = 0; j < c->neighCellNo[i]; ++j) {
        int cellIdx = c->neighCellIdx[(size_t)i * NST + j];
        int ia, ib, id;
        map1Dto3D(c, cellIdx, &ia, &ib, &id);
        if (id < lo || id >= hi) continue;
        const double* wt = &c->neighCellWeight[((size_t)i * NST + j) * 3];
        int64_t f = fidx(c, ia, ib, id);
        c->fx[f] = c->fx[f] - p->fdrag[0] * p->vol * wt[0];
        c->fy[f] = c->fy[f] - p->fdrag[1] * p->vol * wt[1];
        c->fz[f] = c->fz[f] - p->fdrag[2] * p->vol * wt[2];
      }
    }
  }
  return 0;
}

/* FillGhostRegionForFluid (boundary.F90:122-147) for u,v,w on one rank, with
 * the send/recv boxes of BuildMPIRecvAndSendIndexForFluid (boundary.F90:2-108):
 * face by face, the halo beyond face sideRecv takes the cells next to face
 * sideSend (periodic), or, beyond a wall, the mirrored cells next to sideRecv
 * with all three components negated (DealWithBoundaryFluid, boundary.F90:211-245). */
static void face_box(const orc_case* c, int side, int recv, int wall, int lo[3], int hi[3], int inc[3]) {
  int d = side / 2, high = side % 2;
  for (int e = 0; e < 3; ++e) {
    inc[e] = 1;
    if (e < d) { /* axes filled by earlier faces: halo included */
      lo[e] = c->LG[e];
      hi[e] = c->UG[e];
    } else {
      lo[e] = c->SG[e];
      hi[e] = c->EG[e];
    }
  }
  if (!recv) {
    lo[d] = high ? c->EG[d] - HALO + 1 : c->SG[d];
    hi[d] = high ? c->EG[d] : c->SG[d] + HALO - 1;
  } else if (!wall) {
    lo[d] = high ? c->EG[d] + 1 : c->LG[d];
    hi[d] = high ? c->UG[d] : c->SG[d] - 1;
  } else { /* walls fill outward from the face */
    lo[d] = high ? c->UG[d] : c->SG[d] - 1;
    hi[d] = high ? c->EG[d] + 1 : c->LG[d];
    inc[d] = -1;
  }
}
static void FillGhostRegionForFluid(orc_case* c) {
  double* f[3] = {c->u, c->v, c->w};
  for (int i = 0; i < 6; ++i) {
    int sideSend = i, sideRecv = (i % 2 == 0) ? i + 1 : i - 1;
    int wall = c->p.bType[sideRecv] == 1;
    int from = wall ? sideRecv : sideSend; /* DealWithBoundaryFluid reads sendIdxFluid(:,sideRecv) */
    int slo[3], shi[3], sinc[3], rlo[3], rhi[3], rinc[3];
    face_box(c, from, 0, 0, slo, shi, sinc);
    face_box(c, sideRecv, 1, wall, rlo, rhi, rinc);
    int d = sideRecv / 2;
    int nr = (rhi[d] - rlo[d]) * rinc[d] + 1;
    /* the boxes differ only along d; walk both in (k, j, i) order */
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int k = slo[2]; k <= shi[2]; ++k)
      for (int j = slo[1]; j <= shi[1]; ++j)
        for (int ii = slo[0]; ii <= shi[0]; ++ii) {
          int src[3] = {ii, j, k}, dst[3] = {ii, j, k};
          int t = src[d] - slo[d];
          dst[d] = rlo[d] + t * rinc[d];
          if (t >= nr) continue;
          int64_t a = fidx(c, dst[0], dst[1], dst[2]), s0 = fidx(c, src[0], src[1], src[2]);
          for (int q = 0; q < 3; ++q) f[q][a] = wall ? -f[q][s0] : f[q][s0];
        }
  }
}

/* Boundary (fluid.F90:240-249): the wall-normal velocity on the wall face and
 * in the halo beyond it is zero. */
static void Boundary(orc_case* c) {
  double* f[3] = {c->u, c->v, c->w};
  for (int side = 0; side < 6; ++side) {
    if (c->p.bType[side] != 1) continue;
    int d = side / 2;
    int lo[3] = {c->LG[0], c->LG[1], c->LG[2]}, hi[3] = {c->UG[0], c->UG[1], c->UG[2]};
    if (side % 2 == 0) hi[d] = c->SG[d];
    else lo[d] = c->EG[d] + 1;
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) f[d][fidx(c, i, j, k)] = 0.0;
  }
}

/* VelocityPostGuess (fluid.F90:135-153) followed by the halo refill and the
 * wall condition done by FirstOrderForwardEuler (fluid.F90:275-277). */
int orc_VelocityPostGuess(orc_case* c) {
  const double dt = c->p.dt;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int k = c->SG[2]; k <= c->EG[2]; ++k)
    for (int j = c->SG[1]; j <= c->EG[1]; ++j)
      for (int i = c->SG[0]; i <= c->EG[0]; ++i) {
        int64_t f = fidx(c, i, j, k);
        c->u[f] = c->u[f] + dt * (c->fx[f] - c->fxOld[f]);
        c->v[f] = c->v[f] + dt * (c->fy[f] - c->fyOld[f]);
        c->w[f] = c->w[f] + dt * (c->fz[f] - c->fzOld[f]);
      }
  FillGhostRegionForFluid(c);
  Boundary(c);
  return 0;
}

/* ------------------------------------------------------------------ */
/* bodies                                                              */

/* periodic image of the body centre nearest to a marker coordinate
 * (deviation 2); returns the centre itself unless the body straddles. */
static inline double body_ref(const orc_case* c, int d, double xm, double X) {
  double L = c->len[d];
  double diff = xm - X;
  if (diff > 0.5 * L) return X + L;
  if (diff < -0.5 * L) return X - L;
  return X;
}

/* CrossMultiplication (ZJS_AUXILIARY_DEM.F90:20-30) */
static inline void Cross(const double* a, const double* b, double* d) {
  double c1 = a[1] * b[2] - a[2] * b[1];
  double c2 = -a[0] * b[2] + a[2] * b[0];
  double c3 = a[0] * b[1] - a[1] * b[0];
  d[0] = c1;
  d[1] = c2;
  d[2] = c3;
}
/* TensorMultiplication (ZJS_AUXILIARY_DEM.F90:32-48) */
static inline void TensorMul(const double* A, const double* B, double* D) {
  double C[9];
  C[0] = A[0] * B[0] + A[1] * B[3] + A[2] * B[6];
  C[1] = A[0] * B[1] + A[1] * B[4] + A[2] * B[7];
  C[2] = A[0] * B[2] + A[1] * B[5] + A[2] * B[8];
  C[3] = A[3] * B[0] + A[4] * B[3] + A[5] * B[6];
  C[4] = A[3] * B[1] + A[4] * B[4] + A[5] * B[7];
  C[5] = A[3] * B[2] + A[4] * B[5] + A[5] * B[8];
  C[6] = A[6] * B[0] + A[7] * B[3] + A[8] * B[6];
  C[7] = A[6] * B[1] + A[7] * B[4] + A[8] * B[7];
  C[8] = A[6] * B[2] + A[7] * B[5] + A[8] * B[8];
  memcpy(D, C, sizeof C);
}
/* TensorVectorMultiplication (ZJS_AUXILIARY_DEM.F90:50-61) */
static inline void TensorVec(const double* A, const double* b, double* d) {
  double c1 = A[0] * b[0] + A[1] * b[1] + A[2] * b[2];
  double c2 = A[3] * b[0] + A[4] * b[1] + A[5] * b[2];
  double c3 = A[6] * b[0] + A[7] * b[1] + A[8] * b[2];
  d[0] = c1;
  d[1] = c2;
  d[2] = c3;
}
/* InverseOrthogonalMatrix (ZJS_AUXILIARY_DEM.F90:63-72) */
static inline void Transpose(const double* A, double* B) {
  B[0] = A[0]; B[1] = A[3]; B[2] = A[6];
  B[3] = A[1]; B[4] = A[4]; B[5] = A[7];
  B[6] = A[2]; B[7] = A[5]; B[8] = A[8];
}
/* CalculateRotateMatrix (couplesolverCylinder.F90:76-97) */
static void CalculateRotateMatrix(const double* theta, double* mat) {
  double mag = sqrt(theta[0] * theta[0] + theta[1] * theta[1] + theta[2] * theta[2]);
  mag = mag > 1e-10 ? mag : 1e-10;
  double ux = theta[0] / mag, uy = theta[1] / mag, uz = theta[2] / mag;
  double cm = cos(mag), sm = sin(mag);
  mat[0] = (1 - cm) * ux * ux + cm;
  mat[1] = (1 - cm) * ux * uy - sm * uz;
  mat[2] = (1 - cm) * ux * uz + sm * uy;
  mat[3] = (1 - cm) * uy * ux + sm * uz;
  mat[4] = (1 - cm) * uy * uy + cm;
  mat[5] = (1 - cm) * uy * uz - sm * ux;
  mat[6] = (1 - cm) * uz * ux - sm * uy;
  mat[7] = (1 - cm) * uz * uy + sm * ux;
  mat[8] = (1 - cm) * uz * uz + cm;
}

/* AssembleLocalForceMS (ZJS_MS_DEM.F90:494-519), which is all of
 * AssembleForceMS (ZJS_MS_DEM.F90:385-432) on one rank. */
int orc_AssembleLocalForceMS(orc_case* c) {
  for (int b = 0; b < c->nMS; ++b) {
    MultiSphere* B = &c->MS[b];
    memset(B->fdrag, 0, sizeof B->fdrag);
    memset(B->fcol, 0, sizeof B->fcol);
    memset(B->fmom, 0, sizeof B->fmom);
    memset(B->fmomCol, 0, sizeof B->fmomCol);
  }
  const double rhof = c->p.rhof;
  for (int i = 0; i < c->npLocal; ++i) {
    const Parcel* p = &c->part[i];
    if (p->MSIdx < 1 || p->MSIdx > c->nMS) return fail(c, IBMDEM_EINVAL, "parcel %d has MSIdx %d", i + 1, p->MSIdx);
    MultiSphere* B = &c->MS[p->MSIdx - 1];
    for (int k = 0; k < 3; ++k) B->fdrag[k] = B->fdrag[k] + p->fdrag[k] * p->vol * rhof;
    for (int k = 0; k < 3; ++k) B->fcol[k] = B->fcol[k] + p->fcol[k];
    double rpc[3], fv[3], momTmp[3], momCol[3];
    for (int k = 0; k < 3; ++k) rpc[k] = p->x[k] - body_ref(c, k, p->x[k], B->x[k]);
    for (int k = 0; k < 3; ++k) fv[k] = p->fdrag[k] * p->vol;
    Cross(rpc, fv, momTmp);
    Cross(rpc, p->fcol, momCol);
    for (int k = 0; k < 3; ++k) B->fmom[k] = B->fmom[k] + momTmp[k];
    for (int k = 0; k < 3; ++k) B->fmomCol[k] = B->fmomCol[k] + momCol[k];
  }
  return 0;
}

/* EvolutionMS (couplesolverCylinder.F90:2-42) */
int orc_EvolutionMS(orc_case* c) {
  const double dtDEM = c->dtDEM, rhof = c->p.rhof;
  const double* g = c->p.gravity;
  for (int b = 0; b < c->nMS; ++b) {
    MultiSphere* B = &c->MS[b];
    double ratio = (B->rho - rhof) / B->rho;
    memcpy(B->rotMatGloOld, B->rotMatGlo, sizeof B->rotMatGlo);
    for (int k = 0; k < 3; ++k)
      B->v[k] = B->v[k] + B->fhydro[k] * dtDEM + B->fcol[k] / B->m * dtDEM + ratio * g[k] * dtDEM;
    double theta[3] = {B->omega[0] * dtDEM, B->omega[1] * dtDEM, B->omega[2] * dtDEM};
    CalculateRotateMatrix(theta, B->rotMat);
    double ITInv[9], RMInv[9], TMInvTmp[9], TMInv[9];
    memcpy(ITInv, B->InertiaTensor, sizeof ITInv);
    ITInv[0] = 1.0 / ITInv[0];
    ITInv[4] = 1.0 / ITInv[4];
    ITInv[8] = 1.0 / ITInv[8];
    TensorMul(B->rotMatGlo, B->rotMat, B->rotMatGlo);
    Transpose(B->rotMatGlo, RMInv);
    TensorMul(B->rotMatGlo, ITInv, TMInvTmp);
    TensorMul(TMInvTmp, RMInv, TMInv);
    for (int k = 0; k < 3; ++k) B->AngMom[k] = B->AngMom[k] + (B->fmomHydro[k] + B->fmomCol[k]) * dtDEM;
    TensorVec(TMInv, B->AngMom, B->omega);
    for (int k = 0; k < 3; ++k) B->x[k] = B->x[k] + B->v[k] * dtDEM;
  }
  return 0;
}

/* ResetVelocityAndPositionLagrangianPoints (couplesolverCylinder.F90:44-60)
 * with RotateLagrangianPoints (:62-74).  The rotation centre is the periodic
 * image of the body centre nearest the translated marker (deviation 2). */
int orc_ResetVelocityAndPositionLagrangianPoints(orc_case* c) {
  const double dtDEM = c->dtDEM;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int i = 0; i < c->npLocal; ++i) {
    Parcel* p = &c->part[i];
    const MultiSphere* B = &c->MS[p->MSIdx - 1];
    for (int k = 0; k < 3; ++k) p->x[k] = p->x[k] + B->v[k] * dtDEM;
    double xc[3], xt[3];
    for (int k = 0; k < 3; ++k) xc[k] = body_ref(c, k, p->x[k], B->x[k]);
    for (int k = 0; k < 3; ++k) xt[k] = p->x[k] - xc[k];
    const double* m = B->rotMat;
    p->x[0] = m[0] * xt[0] + m[1] * xt[1] + m[2] * xt[2];
    p->x[1] = m[3] * xt[0] + m[4] * xt[1] + m[5] * xt[2];
    p->x[2] = m[6] * xt[0] + m[7] * xt[1] + m[8] * xt[2];
    for (int k = 0; k < 3; ++k) p->x[k] = p->x[k] + xc[k];
    double r[3] = {p->x[0] - xc[0], p->x[1] - xc[1], p->x[2] - xc[2]};
    Cross(B->omega, r, p->v);
    for (int k = 0; k < 3; ++k) p->v[k] = p->v[k] + B->v[k];
  }
  return 0;
}

/* AdjustParcelPosition (ZJS_EVOLUTION_DEM.F90:121-150) */
int orc_AdjustParcelPosition(orc_case* c) {
  double err[3] = {c->di * 1e-20, c->dj * 1e-20, c->dk * 1e-20};
  for (int i = 0; i < c->npLocal; ++i) {
    double* x = c->part[i].x;
    for (int d = 0; d < 3; ++d) {
      if (fabs(x[d] - c->start[d]) < err[d]) x[d] = c->start[d] + err[d];
      if (fabs(x[d] - c->end[d]) < err[d]) x[d] = c->end[d] + err[d];
    }
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* drivers                                                             */

/* tail of InitializationDEM (ZJS_INIT_DEM.F90:24-35) */
int orc_InitializationDEM(orc_case* c) {
  int rc = orc_RebuildAllListOrNot(c);
  if (rc) return rc;
  if ((rc = orc_UpdateLocalCellWeightListDEM(c))) return rc;
  if ((rc = orc_UpdateParcelInfoInGhostRegion(c))) return rc;
  return orc_UpdateGhostCellWeightListDEM(c);
}

/* particle side of FirstOrderForwardEuler (fluid.F90:252-285) */
int orc_MultiDirectForcing(orc_case* c) {
  if (!c->listsBuilt) return fail(c, IBMDEM_ESTATE, "lists not built");
  for (int i = 0; i < c->npLocal; ++i) memset(c->part[i].fdrag, 0, sizeof c->part[i].fdrag);
  size_t nb = (size_t)c->ncell * sizeof(double);
  memset(c->fx, 0, nb);
  memset(c->fy, 0, nb);
  memset(c->fz, 0, nb);
  int rc;
  for (int it = 0; it < c->p.Ns; ++it) {
    if ((rc = orc_UpdateFluidVelocityOnLagrangianPoints(c))) return rc;
    if ((rc = orc_UpdateParcelInfoInGhostRegion(c))) return rc;
    if ((rc = orc_UpdateMomentumSourceTerm(c))) return rc;
    if ((rc = orc_VelocityPostGuess(c))) return rc;
  }
  return 0;
}

/* CloudEvolutionStepMS (couplesolverCylinder.F90:99-187), multi-rank branch */
int orc_CloudEvolutionStepMS(orc_case* c) {
  int rc;
  if ((rc = orc_CalculateCollisionForce(c))) return rc;
  if ((rc = orc_CalculateSolidBoundaryCollisionForce(c))) return rc;
  if ((rc = orc_AssembleLocalForceMS(c))) return rc;
  if ((rc = orc_EvolutionMS(c))) return rc;
  if ((rc = orc_ResetVelocityAndPositionLagrangianPoints(c))) return rc;
  if ((rc = orc_AdjustParcelPosition(c))) return rc;
  if ((rc = orc_UpdateParcelInfoInGhostRegion(c))) return rc;
  if ((rc = orc_RebuildAllListOrNot(c))) return rc;
  if ((rc = orc_UpdateLocalCellWeightListDEM(c))) return rc;
  if ((rc = orc_UpdateParcelInfoInGhostRegion(c))) return rc;
  return orc_UpdateGhostCellWeightListDEM(c);
}

/* CloudEvolutionMS (couplesolverCylinder.F90:189-217) */
int orc_CloudEvolutionMS(orc_case* c) {
  const double dt = c->p.dt, rhof = c->p.rhof;
  for (int b = 0; b < c->nMS; ++b) {
    MultiSphere* B = &c->MS[b];
    memset(B->fhydro, 0, sizeof B->fhydro);
    memset(B->fmomHydro, 0, sizeof B->fmomHydro);
  }
  for (int b = 0; b < c->nMS; ++b) {
    MultiSphere* B = &c->MS[b];
    double ratio = (B->rho - rhof) / B->rho;
    for (int k = 0; k < 3; ++k) B->fhydro[k] = (B->v[k] - B->vold[k]) / dt * (1.0 - ratio);
    for (int k = 0; k < 3; ++k) B->fmomHydro[k] = (B->AngMom[k] - B->AngMomOld[k]) / dt * (1.0 - ratio);
    memcpy(B->vold, B->v, sizeof B->v);
    memcpy(B->AngMomOld, B->AngMom, sizeof B->AngMom);
  }
  int rc = orc_AssembleLocalForceMS(c);
  if (rc) return rc;
  for (int b = 0; b < c->nMS; ++b) {
    MultiSphere* B = &c->MS[b];
    for (int k = 0; k < 3; ++k) B->fhydro[k] = B->fhydro[k] + B->fdrag[k] / B->m;
    for (int k = 0; k < 3; ++k) B->fmomHydro[k] = B->fmomHydro[k] + B->fmom[k];
  }
  for (int s = 0; s < c->p.coupleInterval; ++s)
    if ((rc = orc_CloudEvolutionStepMS(c))) return rc;
  return 0;
}

/* frozen-fluid step: restore u,v,w, then the particle side of one fluid step */
int orc_step(orc_case* c, int32_t nsteps) {
  size_t nb = (size_t)c->ncell * sizeof(double);
  for (int s = 0; s < nsteps; ++s) {
    memcpy(c->u, c->u0, nb);
    memcpy(c->v, c->v0, nb);
    memcpy(c->w, c->w0, nb);
    int rc = orc_MultiDirectForcing(c);
    if (rc) return rc;
    if ((rc = orc_CloudEvolutionMS(c))) return rc;
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* CalculateDragForce (ZJS_DRAGFORCE_DEM.F90:2-35).  Never called by the
 * reference; restated for the unresolved path.  The literals 3.7, 0.65, 0.687,
 * 0.0183, 8.33, 0.0972 are default-real (single precision) in the source. */
void orc_CalculateDragForce(double rho_p, double rad_p, const double* v_p, double denf, double alphaf_local,
                            const double* velf, double* beta) {
  const double c37 = (double)3.7f, c065 = (double)0.65f, c0687 = (double)0.687f, c00183 = (double)0.0183f;
  const double c833 = (double)8.33f, c00972 = (double)0.0972f, c08 = (double)0.8f;
  const double viscf = 1e-5; /* ZJS_VARS.F90:77 */
  double spg = rho_p / denf;
  double diameter = 2.0 * rad_p;
  for (int j = 0; j < 3; ++j) {
    double Ur = fabs(velf[j] - v_p[j]);
    double Rep = Ur * diameter / viscf;
    Rep = Rep > 1.0 ? Rep : 1.0;
    double t = 1.5 - log10(Rep);
    double zeta = c37 - c065 * exp(-0.5 * (t * t));
    double fbase, f;
    if (Rep < 1000)
      fbase = 1 + 1.0 / 6.0 * pow(Rep, c0687);
    else
      fbase = c00183 * Rep;
    if (alphaf_local < c08)
      f = c833 * (1 - alphaf_local) / alphaf_local + c00972 * Rep;
    else
      f = fbase * pow(alphaf_local, -zeta);
    double Cd = 24.0 / Rep * f;
    beta[j] = 0.75 * (Cd * Ur) / (diameter * spg);
  }
}
