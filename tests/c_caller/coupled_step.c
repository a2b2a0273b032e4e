/*
 * A compiled caller of the C ABI, as the reference's Fortran would call it
 * through an ISO_C_BINDING module: plain host arrays in the reference's layout,
 * one call per replaced subroutine.  For each of nsteps fluid steps it does what
 * FirstOrderForwardEuler and the time loop do around the particle side
 * (fluid.F90:252-285, couplesolverCylinder.F90:189-217):
 *
 *   ibmdem_set_fluid(u, v, w)              the solver's current velocity
 *   ibmdem_MultiDirectForcing()            the Ns forcing iterations
 *   ibmdem_get_fluid(u, v, w, fx, fy, fz)  corrected velocity and forcing back
 *   ibmdem_CloudEvolutionMS()              bodies and markers advance
 *
 * and feeds the returned velocity into the next step (a stand-in for the fluid
 * solve between them).  Inputs are raw binary files written by the test
 * (params.bin, parcels.bin, bodies.bin, u.bin, v.bin, w.bin in a directory);
 * outputs are fields.bin (u, v, w, fx, fy, fz), bodies.bin.out and
 * parcels.bin.out.  Usage: coupled_step <dir> <nsteps>.  Exit status 0 on
 * success; on a library error the message is printed and the status is 1.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ibmdem.h"

static void* read_file(const char* dir, const char* name, size_t* bytes) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s", dir, name);
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  void* p = malloc(n > 0 ? (size_t)n : 1);
  if (p && n > 0 && fread(p, 1, (size_t)n, f) != (size_t)n) {
    free(p);
    p = NULL;
  }
  fclose(f);
  *bytes = (size_t)n;
  return p;
}

static int write_file(const char* dir, const char* name, const void* p, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s", dir, name);
  FILE* f = fopen(path, "wb");
  if (!f) return -1;
  size_t w = fwrite(p, 1, bytes, f);
  fclose(f);
  return w == bytes ? 0 : -1;
}

#define CHECK(call)                                                        \
  do {                                                                     \
    int rc_ = (call);                                                      \
    if (rc_ != IBMDEM_OK) {                                                \
      fprintf(stderr, "%s: %d %s\n", #call, rc_, ibmdem_last_error(ctx)); \
      return 1;                                                            \
    }                                                                      \
  } while (0)

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s <dir> <nsteps>\n", argv[0]);
    return 2;
  }
  const char* dir = argv[1];
  const int nsteps = atoi(argv[2]);
  size_t bp = 0, bparts = 0, bbodies = 0, bu = 0, bv = 0, bw = 0;
  ibmdem_params* p = (ibmdem_params*)read_file(dir, "params.bin", &bp);
  ibmdem_parcel* parts = (ibmdem_parcel*)read_file(dir, "parcels.bin", &bparts);
  ibmdem_multisphere* bodies = (ibmdem_multisphere*)read_file(dir, "bodies.bin", &bbodies);
  double* u = (double*)read_file(dir, "u.bin", &bu);
  double* v = (double*)read_file(dir, "v.bin", &bv);
  double* w = (double*)read_file(dir, "w.bin", &bw);
  if (!p || !parts || !bodies || !u || !v || !w || bp != sizeof(ibmdem_params)) {
    fprintf(stderr, "missing or malformed input in %s\n", dir);
    return 2;
  }
  const int32_t np = (int32_t)(bparts / sizeof(ibmdem_parcel));
  const int32_t nb = (int32_t)(bbodies / sizeof(ibmdem_multisphere));
  const size_t nf = bu / sizeof(double);
  if (bv != bu || bw != bu || nf != (size_t)(p->nx + 4) * (p->ny + 4) * (p->nz + 4)) {
    fprintf(stderr, "field size does not match the grid\n");
    return 2;
  }
  ibmdem_ctx* ctx = NULL;
  if (ibmdem_create(p, 0, &ctx) != IBMDEM_OK) {
    fprintf(stderr, "ibmdem_create failed\n");
    return 1;
  }
  CHECK(ibmdem_set_parcels(ctx, np, parts));
  CHECK(ibmdem_set_bodies(ctx, nb, bodies));
  CHECK(ibmdem_set_fluid(ctx, u, v, w));
  CHECK(ibmdem_InitializationDEM(ctx));
  double* f6 = (double*)malloc(6 * nf * sizeof(double));
  if (!f6) return 2;
  double *fu = f6, *fv = f6 + nf, *fw = f6 + 2 * nf, *fx = f6 + 3 * nf, *fy = f6 + 4 * nf, *fz = f6 + 5 * nf;
  for (int s = 0; s < nsteps; ++s) {
    CHECK(ibmdem_set_fluid(ctx, u, v, w));
    CHECK(ibmdem_MultiDirectForcing(ctx));
    CHECK(ibmdem_get_fluid(ctx, fu, fv, fw, fx, fy, fz));
    CHECK(ibmdem_CloudEvolutionMS(ctx));
    memcpy(u, fu, nf * sizeof(double));
    memcpy(v, fv, nf * sizeof(double));
    memcpy(w, fw, nf * sizeof(double));
  }
  int32_t nbOut = 0;
  CHECK(ibmdem_get_bodies(ctx, bodies, nb, &nbOut));
  int32_t nTotal = 0, nLocal = 0;
  CHECK(ibmdem_get_parcels(ctx, NULL, 0, &nTotal, &nLocal));
  ibmdem_parcel* out = (ibmdem_parcel*)malloc((size_t)(nTotal > 0 ? nTotal : 1) * sizeof(ibmdem_parcel));
  if (!out) return 2;
  CHECK(ibmdem_get_parcels(ctx, out, nTotal, &nTotal, &nLocal));
  int rc = write_file(dir, "fields.bin", f6, 6 * nf * sizeof(double));
  rc |= write_file(dir, "bodies.bin.out", bodies, (size_t)nbOut * sizeof(ibmdem_multisphere));
  rc |= write_file(dir, "parcels.bin.out", out, (size_t)nLocal * sizeof(ibmdem_parcel));
  ibmdem_destroy(ctx);
  printf("steps %d parcels %d locals %d bodies %d\n", nsteps, nTotal, nLocal, nbOut);
  return rc ? 2 : 0;
}
