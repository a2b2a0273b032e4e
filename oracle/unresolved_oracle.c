/*
 * unresolved_oracle.c — CPU restatement of the unresolved CFD-DEM path.
 *
 * TEST INFRASTRUCTURE ONLY (parity reference and timed CPU baseline); the
 * product never links or calls it.
 *
 * PARITY UNPINNED beyond the drag law: the reference holds only the drag law
 * of this path (CalculateDragForce, ZJS_DRAGFORCE_DEM.F90:2-35, restated in
 * orc_CalculateDragForce and pinned bit for bit to the reference's own
 * subroutine by tests/test_reference_pins.py), the normal contact law it shares with the resolved
 * path (ZJS_COLLISION_DEM.F90:30-57) and an empty LogVolumeFraction
 * (ZJS_EVOLUTION_DEM.F90:27-32).  The rest -- tangential friction with history,
 * the Gaussian volume fraction, interpolation at the particle and the
 * integrator -- is the definition written in include/ibmdem.h, restated here
 * with the same loop and evaluation order as the CUDA path, and pinned by the
 * analytic checks in tests/test_oracle_unresolved.py.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ibmdem_oracle.h"

enum { F_RAD = 0, F_RHO, F_VOL, F_M, F_I, F_X, F_V = F_X + 3, F_W = F_V + 3, F_FCOL = F_W + 3, F_TCOL = F_FCOL + 3,
       F_FDRAG = F_TCOL + 3, F_ALPHA = F_FDRAG + 3, F_ND };

struct orc_ucase {
  ibmdem_uparams p;
  int n[3], ni, nj, nc[3], K;
  long long nint, ncd;
  double h, vcell, L[3], halfL[3], cs[3], eta;
  int np;
  double* d;  /* F_ND * np, field-major */
  int* gidx;
  double *uf, *vf, *wf, *alphaf;
  int *ncOld, *pOld, *ncNew, *pNew;
  double *xOld, *xNew;
  int *demStart, *demItems, *flStart, *flItems;
  double* gw;
  int stepped;
  char err[256];
};

static int ufail(orc_ucase* u, int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(u->err, sizeof u->err, fmt, ap);
  va_end(ap);
  return code;
}

#define D(f, i) u->d[(size_t)(f) * u->np + (i)]

static double eta_of(double e) {
  /* ZJS_COLLISION_DEM.F90:30: 3.1415926536 is a single-precision literal */
  float pi32 = 3.1415926536f;
  float pi2 = pi32 * pi32;
  return -2 * log(e) / sqrt((double)pi2 + log(e));
}

orc_ucase* orc_u_create(const ibmdem_uparams* p) {
  if (!p || p->nx < 5 || p->ny < 5 || p->nz < 5 || !(p->dx > 0) || !(p->dcell > 0) || p->maxContacts < 1) return NULL;
  orc_ucase* u = calloc(1, sizeof *u);
  if (!u) return NULL;
  u->p = *p;
  u->n[0] = p->nx;
  u->n[1] = p->ny;
  u->n[2] = p->nz;
  u->ni = p->nx + 4;
  u->nj = p->ny + 4;
  u->nint = (long long)p->nx * p->ny * p->nz;
  u->h = p->dx;
  u->vcell = p->dx * p->dx * p->dx;
  u->ncd = 1;
  for (int d = 0; d < 3; ++d) {
    u->L[d] = p->dx * u->n[d];
    u->halfL[d] = 0.5 * u->L[d];
    int c = (int)floor(u->L[d] / p->dcell);
    u->nc[d] = c < 3 ? 3 : c;
    u->cs[d] = u->L[d] / u->nc[d];
    u->ncd *= u->nc[d];
  }
  u->K = p->maxContacts;
  u->eta = eta_of(p->ResistCoeff);
  size_t nf = (size_t)u->ni * u->nj * (p->nz + 4);
  u->uf = calloc(nf, sizeof(double));
  u->vf = calloc(nf, sizeof(double));
  u->wf = calloc(nf, sizeof(double));
  u->alphaf = calloc((size_t)u->nint, sizeof(double));
  u->demStart = calloc((size_t)u->ncd + 1, sizeof(int));
  u->flStart = calloc((size_t)u->nint + 1, sizeof(int));
  snprintf(u->err, sizeof u->err, "ok");
  return u;
}

static void free_particles(orc_ucase* u) {
  void* ps[] = {u->d, u->gidx, u->ncOld, u->pOld, u->ncNew, u->pNew, u->xOld, u->xNew, u->demItems, u->flItems, u->gw};
  for (size_t k = 0; k < sizeof ps / sizeof ps[0]; ++k) free(ps[k]);
  u->d = NULL;
  u->gidx = u->ncOld = u->pOld = u->ncNew = u->pNew = u->demItems = u->flItems = NULL;
  u->xOld = u->xNew = u->gw = NULL;
  u->np = 0;
}

void orc_u_destroy(orc_ucase* u) {
  if (!u) return;
  free_particles(u);
  free(u->uf);
  free(u->vf);
  free(u->wf);
  free(u->alphaf);
  free(u->demStart);
  free(u->flStart);
  free(u);
}

const char* orc_u_last_error(const orc_ucase* u) { return u ? u->err : "null case"; }

int orc_u_set_fluid(orc_ucase* u, const double* uf, const double* vf, const double* wf) {
  size_t nf = (size_t)u->ni * u->nj * (u->p.nz + 4);
  memcpy(u->uf, uf, nf * sizeof(double));
  memcpy(u->vf, vf, nf * sizeof(double));
  memcpy(u->wf, wf, nf * sizeof(double));
  return 0;
}

int orc_u_set_particles(orc_ucase* u, int32_t np, const ibmdem_particle* parts) {
  for (int i = 0; i < np; ++i)
    for (int d = 0; d < 3; ++d)
      if (!(parts[i].x[d] >= 0.0 && parts[i].x[d] < u->L[d]))
        return ufail(u, IBMDEM_ERANGE, "particle %d is outside the periodic box", i);
  free_particles(u);
  u->np = np;
  size_t n = np > 0 ? (size_t)np : 1, K = (size_t)u->K;
  u->d = calloc((size_t)F_ND * n, sizeof(double));
  u->gidx = calloc(n, sizeof(int));
  u->ncOld = calloc(n, sizeof(int));
  u->ncNew = calloc(n, sizeof(int));
  u->pOld = calloc(n * K, sizeof(int));
  u->pNew = calloc(n * K, sizeof(int));
  u->xOld = calloc(3 * n * K, sizeof(double));
  u->xNew = calloc(3 * n * K, sizeof(double));
  u->demItems = calloc(n, sizeof(int));
  u->flItems = calloc(n, sizeof(int));
  u->gw = calloc(16 * n, sizeof(double));
  for (int i = 0; i < np; ++i) {
    const ibmdem_particle* q = &parts[i];
    D(F_RAD, i) = q->rad;
    D(F_RHO, i) = q->rho;
    D(F_VOL, i) = q->vol;
    D(F_M, i) = q->m;
    D(F_I, i) = q->I;
    for (int d = 0; d < 3; ++d) {
      D(F_X + d, i) = q->x[d];
      D(F_V + d, i) = q->v[d];
      D(F_W + d, i) = q->omega[d];
      D(F_FCOL + d, i) = q->fcol[d];
      D(F_TCOL + d, i) = q->tcol[d];
      D(F_FDRAG + d, i) = q->fdrag[d];
    }
    D(F_ALPHA, i) = q->alphaf;
    u->gidx[i] = q->globalIdx;
  }
  u->stepped = 0;
  return 0;
}

int orc_u_get_particles(orc_ucase* u, ibmdem_particle* parts, int32_t cap, int32_t* n) {
  if (n) *n = u->np;
  if (!parts) return 0;
  for (int i = 0; i < u->np && i < cap; ++i) {
    ibmdem_particle* q = &parts[i];
    memset(q, 0, sizeof *q);
    q->globalIdx = u->gidx[i];
    q->rad = D(F_RAD, i);
    q->rho = D(F_RHO, i);
    q->vol = D(F_VOL, i);
    q->m = D(F_M, i);
    q->I = D(F_I, i);
    for (int d = 0; d < 3; ++d) {
      q->x[d] = D(F_X + d, i);
      q->v[d] = D(F_V + d, i);
      q->omega[d] = D(F_W + d, i);
      q->fcol[d] = D(F_FCOL + d, i);
      q->tcol[d] = D(F_TCOL + d, i);
      q->fdrag[d] = D(F_FDRAG + d, i);
    }
    q->alphaf = D(F_ALPHA, i);
  }
  return 0;
}

int orc_u_get_volume_fraction(orc_ucase* u, double* alphaf) {
  if (!u->stepped) return ufail(u, IBMDEM_ESTATE, "no step has run");
  memcpy(alphaf, u->alphaf, sizeof(double) * (size_t)u->nint);
  return 0;
}

int orc_u_get_contacts(orc_ucase* u, int32_t* start, int32_t* partner, double* xi, int32_t* ncontacts) {
  int tot = 0;
  for (int i = 0; i < u->np; ++i) {
    if (start) start[i] = tot;
    for (int s = 0; s < u->ncOld[i]; ++s) {
      if (partner) partner[tot] = u->pOld[(size_t)i * u->K + s];
      if (xi)
        for (int d = 0; d < 3; ++d) xi[3 * (size_t)tot + d] = u->xOld[((size_t)i * u->K + s) * 3 + d];
      ++tot;
    }
  }
  if (start) start[u->np] = tot;
  if (ncontacts) *ncontacts = tot;
  return 0;
}

static int dem_axis(const orc_ucase* u, int d, double x) {
  int c = (int)floor(x / u->cs[d]);
  if (c < 0) c = 0;
  if (c > u->nc[d] - 1) c = u->nc[d] - 1;
  return c;
}

static double min_image(double d, double L, double halfL) {
  if (d > halfL) return d - L;
  if (d < -halfL) return d + L;
  return d;
}

/* stable counting sort of particles by key into CSR (start[nkeys+1], items) */
static void csr_by_key(int np, const long long* key, long long nkeys, int* start, int* items) {
  memset(start, 0, sizeof(int) * (size_t)(nkeys + 1));
  for (int i = 0; i < np; ++i) start[key[i] + 1]++;
  for (long long k = 0; k < nkeys; ++k) start[k + 1] += start[k];
  int* fill = malloc(sizeof(int) * (size_t)(nkeys > 0 ? nkeys : 1));
  memcpy(fill, start, sizeof(int) * (size_t)nkeys);
  for (int i = 0; i < np; ++i) items[fill[key[i]]++] = i;
  free(fill);
}

/* CalculateDragForce with the case's viscf (ZJS_DRAGFORCE_DEM.F90:2-35) */
static void beta_of(double rho_p, double rad_p, const double* v_p, double denf, double alphaf_local, const double* velf,
                    double viscf, double* beta) {
  const double c37 = (double)3.7f, c065 = (double)0.65f, c0687 = (double)0.687f, c00183 = (double)0.0183f;
  const double c833 = (double)8.33f, c00972 = (double)0.0972f, c08 = (double)0.8f;
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

static double lerp3(const orc_ucase* u, const double* F, int i0, int j0, int k0, double tx, double ty, double tz) {
#define AT(i, j, k) F[((long long)((k) + 1) * u->nj + ((j) + 1)) * u->ni + ((i) + 1)]
  double sx = 1.0 - tx, sy = 1.0 - ty, sz = 1.0 - tz;
  double c00 = AT(i0, j0, k0) * sx + AT(i0 + 1, j0, k0) * tx;
  double c10 = AT(i0, j0 + 1, k0) * sx + AT(i0 + 1, j0 + 1, k0) * tx;
  double c01 = AT(i0, j0, k0 + 1) * sx + AT(i0 + 1, j0, k0 + 1) * tx;
  double c11 = AT(i0, j0 + 1, k0 + 1) * sx + AT(i0 + 1, j0 + 1, k0 + 1) * tx;
#undef AT
  double c0 = c00 * sy + c10 * ty;
  double c1 = c01 * sy + c11 * ty;
  return c0 * sz + c1 * tz;
}

static int one_step(orc_ucase* u) {
  const int np = u->np, K = u->K;
  const ibmdem_uparams* p = &u->p;
  long long* kd = malloc(sizeof(long long) * (size_t)(np > 0 ? np : 1));
  long long* kf = malloc(sizeof(long long) * (size_t)(np > 0 ? np : 1));
  for (int i = 0; i < np; ++i) {
    int cd[3], cf[3];
    for (int d = 0; d < 3; ++d) {
      double x = D(F_X + d, i);
      if (!(x >= 0.0 && x < u->L[d])) {
        free(kd);
        free(kf);
        return ufail(u, IBMDEM_ERANGE, "particle %d is outside the periodic box", i);
      }
      cd[d] = dem_axis(u, d, x);
      int f = (int)floor(x / u->h);
      cf[d] = f < 0 ? 0 : (f > u->n[d] - 1 ? u->n[d] - 1 : f);
    }
    kd[i] = ((long long)cd[2] * u->nc[1] + cd[1]) * u->nc[0] + cd[0];
    kf[i] = ((long long)cf[2] * u->n[1] + cf[1]) * u->n[0] + cf[0];
  }
  csr_by_key(np, kd, u->ncd, u->demStart, u->demItems);
  csr_by_key(np, kf, u->nint, u->flStart, u->flItems);
  free(kd);
  free(kf);
  int overflow = -1;

  /* contacts, tangential history and the contact force and torque */
#pragma omp parallel for schedule(dynamic, 256) num_threads(orc_get_threads())
  for (int i = 0; i < np; ++i) {
    const double xi0 = D(F_X, i), xi1 = D(F_X + 1, i), xi2 = D(F_X + 2, i);
    const double vi0 = D(F_V, i), vi1 = D(F_V + 1, i), vi2 = D(F_V + 2, i);
    const double wi0 = D(F_W, i), wi1 = D(F_W + 1, i), wi2 = D(F_W + 2, i);
    const double mi = D(F_M, i), ri = D(F_RAD, i);
    const int c0 = dem_axis(u, 0, xi0), c1 = dem_axis(u, 1, xi1), c2 = dem_axis(u, 2, xi2);
    double f0 = 0, f1 = 0, f2 = 0, t0 = 0, t1 = 0, t2 = 0;
    int m = 0;
    for (int dz = -1; dz <= 1; ++dz) {
      int cz = (c2 + dz + u->nc[2]) % u->nc[2];
      for (int dy = -1; dy <= 1; ++dy) {
        int cy = (c1 + dy + u->nc[1]) % u->nc[1];
        for (int dx = -1; dx <= 1; ++dx) {
          int cx = (c0 + dx + u->nc[0]) % u->nc[0];
          long long cell = ((long long)cz * u->nc[1] + cy) * u->nc[0] + cx;
          for (int q = u->demStart[cell]; q < u->demStart[cell + 1]; ++q) {
            int j = u->demItems[q];
            if (j == i) continue;
            double r1 = min_image(xi0 - D(F_X, j), u->L[0], u->halfL[0]);
            double r2 = min_image(xi1 - D(F_X + 1, j), u->L[1], u->halfL[1]);
            double r3 = min_image(xi2 - D(F_X + 2, j), u->L[2], u->halfL[2]);
            double rj = D(F_RAD, j);
            double rij = ri + rj;
            double d2 = r1 * r1 + r2 * r2 + r3 * r3;
            if (!(d2 < rij * rij)) continue;
            double dist = sqrt(d2);
            double n1 = r1 / dist, n2 = r2 / dist, n3 = r3 / dist;
            double mj = D(F_M, j);
            double meff = 2 * mi * mj / (mi + mj);
            double deltan = rij - dist;
            double kn = p->knCoeff / (0.1 * u->h) * meff;
            double etan = u->eta * sqrt(meff * kn);
            double u1 = vi0 - D(F_V, j), u2 = vi1 - D(F_V + 1, j), u3 = vi2 - D(F_V + 2, j);
            double vn = n1 * u1 + n2 * u2 + n3 * u3;
            double fn = kn * deltan - etan * vn;
            double s1 = ri * wi0 + rj * D(F_W, j);
            double s2 = ri * wi1 + rj * D(F_W + 1, j);
            double s3 = ri * wi2 + rj * D(F_W + 2, j);
            double vr1 = u1 - (s2 * n3 - s3 * n2);
            double vr2 = u2 - (s3 * n1 - s1 * n3);
            double vr3 = u3 - (s1 * n2 - s2 * n1);
            double vrn = n1 * vr1 + n2 * vr2 + n3 * vr3;
            double vt1 = vr1 - vrn * n1, vt2 = vr2 - vrn * n2, vt3 = vr3 - vrn * n3;
            double h1 = 0, h2 = 0, h3 = 0;
            for (int s = 0; s < u->ncOld[i]; ++s)
              if (u->pOld[(size_t)i * K + s] == j) {
                const double* o = u->xOld + ((size_t)i * K + s) * 3;
                h1 = o[0];
                h2 = o[1];
                h3 = o[2];
                break;
              }
            double hn = n1 * h1 + n2 * h2 + n3 * h3;
            h1 = h1 - hn * n1;
            h2 = h2 - hn * n2;
            h3 = h3 - hn * n3;
            h1 = h1 + p->dt * vt1;
            h2 = h2 + p->dt * vt2;
            h3 = h3 + p->dt * vt3;
            double kt = p->ktRatio * kn;
            double etat = u->eta * sqrt(meff * kt);
            double ft1 = -kt * h1 - etat * vt1, ft2 = -kt * h2 - etat * vt2, ft3 = -kt * h3 - etat * vt3;
            double ftm = sqrt(ft1 * ft1 + ft2 * ft2 + ft3 * ft3);
            double lim = p->mu * fabs(fn);
            if (ftm > lim) {
              double sc = lim / ftm;
              ft1 = ft1 * sc;
              ft2 = ft2 * sc;
              ft3 = ft3 * sc;
              h1 = -(ft1 + etat * vt1) / kt;
              h2 = -(ft2 + etat * vt2) / kt;
              h3 = -(ft3 + etat * vt3) / kt;
            }
            f0 = f0 + (fn * n1 + ft1);
            f1 = f1 + (fn * n2 + ft2);
            f2 = f2 + (fn * n3 + ft3);
            t0 = t0 - ri * (n2 * ft3 - n3 * ft2);
            t1 = t1 - ri * (n3 * ft1 - n1 * ft3);
            t2 = t2 - ri * (n1 * ft2 - n2 * ft1);
            if (m < K) {
              u->pNew[(size_t)i * K + m] = j;
              double* o = u->xNew + ((size_t)i * K + m) * 3;
              o[0] = h1;
              o[1] = h2;
              o[2] = h3;
            } else {
#pragma omp critical
              if (overflow < 0) overflow = i;
            }
            ++m;
          }
        }
      }
    }
    u->ncNew[i] = m < K ? m : K;
    D(F_FCOL, i) = f0;
    D(F_FCOL + 1, i) = f1;
    D(F_FCOL + 2, i) = f2;
    D(F_TCOL, i) = t0;
    D(F_TCOL + 1, i) = t1;
    D(F_TCOL + 2, i) = t2;
  }
  if (overflow >= 0) return ufail(u, IBMDEM_ECAPACITY, "particle %d touches more than %d partners", overflow, K);

  /* Gaussian weights per particle */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int i = 0; i < np; ++i) {
    double sigma = p->bandwidth * (2.0 * D(F_RAD, i));
    double sum[3];
    double* o = u->gw + (size_t)i * 16;
    for (int d = 0; d < 3; ++d) {
      double x = D(F_X + d, i);
      int a = (int)floor(x / u->h);
      a = a < 0 ? 0 : (a > u->n[d] - 1 ? u->n[d] - 1 : a);
      double s = 0.0;
      for (int q = 0; q < 5; ++q) {
        double xc = ((double)(a - 2 + q) + 0.5) * u->h;
        double t = (x - xc) / sigma;
        double w = exp(-0.5 * (t * t));
        o[d * 5 + q] = w;
        s = s + w;
      }
      sum[d] = s;
    }
    o[15] = D(F_VOL, i) / (((sum[0] * sum[1]) * sum[2]) * u->vcell);
  }

  /* solid volume fraction, gathered per fluid cell from the partial sums of the
     125 source cells around it (z outermost) */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (long long c = 0; c < u->nint; ++c) {
    int i = (int)(c % u->n[0]);
    int j = (int)((c / u->n[0]) % u->n[1]);
    int k = (int)(c / ((long long)u->n[0] * u->n[1]));
    double ap = 0.0;
    for (int oz = -2; oz <= 2; ++oz) {
      int sz = (k + oz + u->n[2]) % u->n[2];
      for (int oy = -2; oy <= 2; ++oy) {
        int sy = (j + oy + u->n[1]) % u->n[1];
        for (int ox = -2; ox <= 2; ++ox) {
          int sx = (i + ox + u->n[0]) % u->n[0];
          long long src = ((long long)sz * u->n[1] + sy) * u->n[0] + sx;
          /* the source cell's partial sum over its particles in part order */
          double t = 0.0;
          for (int q = u->flStart[src]; q < u->flStart[src + 1]; ++q) {
            const double* w = u->gw + (size_t)u->flItems[q] * 16;
            t = t + ((w[15] * w[10 + 2 - oz]) * w[5 + 2 - oy]) * w[2 - ox];
          }
          ap = ap + t;
        }
      }
    }
    double af = 1.0 - ap;
    u->alphaf[c] = af > p->alphaMin ? af : p->alphaMin;
  }

  /* fluid velocity and fraction at the particle, drag, time step */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int i = 0; i < np; ++i) {
    double x[3], v[3], vel[3];
    for (int d = 0; d < 3; ++d) {
      x[d] = D(F_X + d, i);
      v[d] = D(F_V + d, i);
    }
    const double* F[3] = {u->uf, u->vf, u->wf};
    for (int c = 0; c < 3; ++c) {
      int i0[3];
      double t[3];
      for (int d = 0; d < 3; ++d) {
        double f = x[d] / u->h + (d == c ? 1.0 : 0.5);
        i0[d] = (int)floor(f);
        t[d] = f - (double)i0[d];
      }
      vel[c] = lerp3(u, F[c], i0[0], i0[1], i0[2], t[0], t[1], t[2]);
    }
    int a0[3];
    double ta[3];
    for (int d = 0; d < 3; ++d) {
      double f = x[d] / u->h - 0.5;
      a0[d] = (int)floor(f);
      ta[d] = f - (double)a0[d];
    }
#define A(di, dj, dk)                                                                            \
  u->alphaf[((long long)((a0[2] + (dk) + u->n[2]) % u->n[2]) * u->n[1] +                        \
             ((a0[1] + (dj) + u->n[1]) % u->n[1])) * u->n[0] + ((a0[0] + (di) + u->n[0]) % u->n[0])]
    double sx = 1.0 - ta[0], sy = 1.0 - ta[1], sz = 1.0 - ta[2];
    double c00 = A(0, 0, 0) * sx + A(1, 0, 0) * ta[0];
    double c10 = A(0, 1, 0) * sx + A(1, 1, 0) * ta[0];
    double c01 = A(0, 0, 1) * sx + A(1, 0, 1) * ta[0];
    double c11 = A(0, 1, 1) * sx + A(1, 1, 1) * ta[0];
#undef A
    double af = (c00 * sy + c10 * ta[1]) * sz + (c01 * sy + c11 * ta[1]) * ta[2];
    double beta[3];
    double m = D(F_M, i), rho = D(F_RHO, i), I = D(F_I, i);
    beta_of(rho, D(F_RAD, i), v, p->rhof, af, vel, p->viscf, beta);
    double ratio = 1.0 - p->rhof / rho;
    for (int d = 0; d < 3; ++d) {
      double fd = (m * beta[d]) * (vel[d] - v[d]);
      D(F_FDRAG + d, i) = fd;
      double a = (fd + D(F_FCOL + d, i)) / m;
      a = a + ratio * p->gravity[d];
      double vn = v[d] + p->dt * a;
      D(F_V + d, i) = vn;
      D(F_W + d, i) = D(F_W + d, i) + p->dt * (D(F_TCOL + d, i) / I);
      double xn = x[d] + p->dt * vn;
      if (xn >= u->L[d])
        xn = xn + (-u->L[d]);
      else if (xn < 0.0)
        xn = xn + u->L[d];
      D(F_X + d, i) = xn;
    }
    D(F_ALPHA, i) = af;
  }
  /* the new history becomes the old one */
  int* ti = u->ncOld;
  u->ncOld = u->ncNew;
  u->ncNew = ti;
  ti = u->pOld;
  u->pOld = u->pNew;
  u->pNew = ti;
  double* td = u->xOld;
  u->xOld = u->xNew;
  u->xNew = td;
  u->stepped = 1;
  return 0;
}

int orc_u_step(orc_ucase* u, int32_t nsteps) {
  for (int s = 0; s < nsteps; ++s) {
    int rc = one_step(u);
    if (rc) return rc;
  }
  return 0;
}
