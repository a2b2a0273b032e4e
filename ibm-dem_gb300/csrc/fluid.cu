// fluid.cu — the fluid stencils of FirstOrderForwardEuler around the Poisson
// solve (fluid.F90:2-249) and the fluid halo fill (boundary.F90:122-247) on
// the context's device fields.
//
// Every statement keeps the reference's operations in the reference's order
// (FP64, no contraction: -fmad=false), so the fields are bit-identical to a
// serial run of the Fortran, except ModifyBulkVelocity's interior sums, which
// are formed in a fixed order of their own.  Divisions by dt, rhof and the
// Runge-Kutta coefficient are correctly rounded products with a split
// reciprocal (div_split); by a unit spacing they are skipped.  One thread per interior node;
// the stencil neighbours come through L1/L2, so each kernel streams its
// fields about once from HBM.
#include <algorithm>
#include <string>

#include "common.cuh"
#include "kernels.cuh"

namespace ibmdem {

namespace {

constexpr int kFBlock = 256;
constexpr int kSumBlocks = 1024;  // blocks of the ordered interior sums

// interior node t (i fastest) -> (i, j, k), 1-based
__device__ inline void interior_ijk(const Geom& g, uint32_t t, int& i, int& j, int& k) {
  const uint32_t row = g.fdN0.div(t);
  const uint32_t kk = g.fdN1.div(row);
  i = (int)(t - row * (uint32_t)g.n[0]) + 1;
  j = (int)(row - kk * (uint32_t)g.n[1]) + 1;
  k = (int)kk + 1;
}

// x / h for a grid spacing: with unit spacing the division by 1.0 (or by
// 1.0*1.0) is an identity and is skipped
template <bool UNIT>
__device__ inline double by_h(double x, double h) {
  return UNIT ? x : x / h;
}

struct FluidPtrs {
  const double *u, *v, *w, *P, *fx, *fy, *fz, *uold, *vold, *wold;
  double *nu, *nv, *nw, *Px, *Py, *Pz, *RHSul, *RHSvl, *RHSwl;
};

// x is zero or its exponent keeps x/4 normal and x*4 finite
__device__ inline bool scalable(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)(b >> 52) & 0x7ff;
  return (b << 1) == 0 || (e >= 3 && e <= 2044);
}

// The reference's difference of two fluxes on opposite faces,
// 0.5*s1*0.5*t1 - 0.5*s2*0.5*t2 (each product left to right).  When s1, s2,
// the products and their difference are zero or far from the subnormal and
// overflow ranges, the factors 0.5*0.5 are an exact scaling by 1/4 that
// commutes with every rounding, so the value is 0.25*RN(RN(s1*t1) - RN(s2*t2))
// bit for bit; otherwise the statement is evaluated as written.
__device__ inline double flux_diff(double s1, double t1, double s2, double t2) {
  const double p1 = s1 * t1, p2 = s2 * t2, d = p1 - p2;
  if (scalable(s1) && scalable(s2) && scalable(p1) && scalable(p2) && scalable(d)) return d * 0.25;
  return 0.5 * s1 * 0.5 * t1 - 0.5 * s2 * 0.5 * t2;
}

// VelocityGuess (fluid.F90:108-133) with ConvectionTensor (fluid.F90:2-54),
// ViscousTensor (fluid.F90:56-76) and PressureGradient (fluid.F90:78-91).
// A1, C1: aRK == 1, cRK == 1, whose products are identities.
template <bool UNIT, bool A1, bool C1>
__global__ void __launch_bounds__(kFBlock) k_velocity_guess(Geom g, FluidPtrs f, double aRK, double bRK, double cRK,
                                                           double visc, double CPx, double CPy, double CPz) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint32_t)g.nint) return;
  int i, j, k;
  interior_ijk(g, t, i, j, k);
  const long long sj = g.ni, sk = (long long)g.ni * g.nj;
  const long long c = field_off(g, i, j, k);
  const double *u = f.u, *v = f.v, *w = f.w;
  const double dx = g.h[0], dy = g.h[1], dz = g.h[2], dt = g.dt;
  // 2nd order centre differences of the fluxes on the control-volume faces:
  // uuE - uuW, uvB - uvF, ... (fluid.F90:15-33)
  const double TIux = by_h<UNIT>(flux_diff(u[c + 1] + u[c], u[c + 1] + u[c], u[c - 1] + u[c], u[c - 1] + u[c]), dx);
  const double TIuy = by_h<UNIT>(
      flux_diff(u[c + sj] + u[c], v[c - 1 + sj] + v[c + sj], u[c - sj] + u[c], v[c - 1] + v[c]), dy);
  const double TIuz = by_h<UNIT>(
      flux_diff(u[c + sk] + u[c], w[c - 1 + sk] + w[c + sk], u[c - sk] + u[c], w[c - 1] + w[c]), dz);
  const double TIvx = by_h<UNIT>(
      flux_diff(v[c + 1] + v[c], u[c + 1 - sj] + u[c + 1], v[c - 1] + v[c], u[c - sj] + u[c]), dx);
  const double TIvy = by_h<UNIT>(
      flux_diff(v[c + sj] + v[c], v[c + sj] + v[c], v[c - sj] + v[c], v[c - sj] + v[c]), dy);
  const double TIvz = by_h<UNIT>(
      flux_diff(v[c + sk] + v[c], w[c - sj + sk] + w[c + sk], v[c - sk] + v[c], w[c - sj] + w[c]), dz);
  const double TIwx = by_h<UNIT>(
      flux_diff(w[c + 1] + w[c], u[c + 1 - sk] + u[c + 1], w[c - 1] + w[c], u[c - sk] + u[c]), dx);
  const double TIwy = by_h<UNIT>(
      flux_diff(w[c + sj] + w[c], v[c + sj - sk] + v[c + sj], w[c - sj] + w[c], v[c - sk] + v[c]), dy);
  const double TIwz = by_h<UNIT>(
      flux_diff(w[c + sk] + w[c], w[c + sk] + w[c], w[c - sk] + w[c], w[c - sk] + w[c]), dz);

  const double TVux = by_h<UNIT>(u[c + 1] + u[c - 1] - 2.0 * u[c], dx * dx) * visc;
  const double TVuy = by_h<UNIT>(u[c + sj] + u[c - sj] - 2.0 * u[c], dy * dy) * visc;
  const double TVuz = by_h<UNIT>(u[c + sk] + u[c - sk] - 2.0 * u[c], dz * dz) * visc;
  const double TVvx = by_h<UNIT>(v[c + 1] + v[c - 1] - 2.0 * v[c], dx * dx) * visc;
  const double TVvy = by_h<UNIT>(v[c + sj] + v[c - sj] - 2.0 * v[c], dy * dy) * visc;
  const double TVvz = by_h<UNIT>(v[c + sk] + v[c - sk] - 2.0 * v[c], dz * dz) * visc;
  const double TVwx = by_h<UNIT>(w[c + 1] + w[c - 1] - 2.0 * w[c], dx * dx) * visc;
  const double TVwy = by_h<UNIT>(w[c + sj] + w[c - sj] - 2.0 * w[c], dy * dy) * visc;
  const double TVwz = by_h<UNIT>(w[c + sk] + w[c - sk] - 2.0 * w[c], dz * dz) * visc;

  const double* P = f.P;
  const double Px = div_split(by_h<UNIT>(P[c] - P[c - 1], dx), g.srhof);
  const double Py = div_split(by_h<UNIT>(P[c] - P[c - sj], dy), g.srhof);
  const double Pz = div_split(by_h<UNIT>(P[c] - P[c - sk], dz), g.srhof);

  const double RHSu = -(TIux + TIuy + TIuz) + (TVux + TVuy + TVuz) + CPx + f.fx[c];
  const double RHSv = -(TIvx + TIvy + TIvz) + (TVvx + TVvy + TVvz) + CPy + f.fy[c];
  const double RHSw = -(TIwx + TIwy + TIwz) + (TVwx + TVwy + TVwz) + CPz + f.fz[c];
  // aRK*RHS and cRK*grad P with a coefficient of 1 are the values themselves
  f.nu[c] = f.uold[c] + dt * ((A1 ? RHSu : aRK * RHSu) + bRK * f.RHSul[c] - (C1 ? Px : cRK * Px));
  f.nv[c] = f.vold[c] + dt * ((A1 ? RHSv : aRK * RHSv) + bRK * f.RHSvl[c] - (C1 ? Py : cRK * Py));
  f.nw[c] = f.wold[c] + dt * ((A1 ? RHSw : aRK * RHSw) + bRK * f.RHSwl[c] - (C1 ? Pz : cRK * Pz));
  f.Px[c] = Px;
  f.Py[c] = Py;
  f.Pz[c] = Pz;
  // RHSul = RHSu after the loop (fluid.F90:130-132); no node reads another's
  f.RHSul[c] = RHSu;
  f.RHSvl[c] = RHSv;
  f.RHSwl[c] = RHSw;
}

// the guess's interior values into u,v,w (the stencils above read the old ones)
__global__ void k_copy_interior3(Geom g, const double* nu, const double* nv, const double* nw, double* u, double* v,
                                 double* w) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint32_t)g.nint) return;
  int i, j, k;
  interior_ijk(g, t, i, j, k);
  const long long c = field_off(g, i, j, k);
  u[c] = nu[c];
  v[c] = nv[c];
  w[c] = nw[c];
}

// VelocityDivergence (fluid.F90:93-106)
template <bool UNIT>
__global__ void k_velocity_divergence(Geom g, const double* u, const double* v, const double* w, double* velDiv,
                                      SplitRecip cRK) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint32_t)g.nint) return;
  int i, j, k;
  interior_ijk(g, t, i, j, k);
  const long long sj = g.ni, sk = (long long)g.ni * g.nj;
  const long long c = field_off(g, i, j, k);
  const double d = by_h<UNIT>(u[c + 1] - u[c], g.h[0]) + by_h<UNIT>(v[c + sj] - v[c], g.h[1]) +
                   by_h<UNIT>(w[c + sk] - w[c], g.h[2]);
  velDiv[c] = div_split(div_split(-d, g.sdt), cRK) * g.rhof;
}

// PressureCorrection (fluid.F90:197-208)
__global__ void k_pressure_correction(Geom g, double* P, const double* Pcorr) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint32_t)g.nint) return;
  int i, j, k;
  interior_ijk(g, t, i, j, k);
  const long long c = field_off(g, i, j, k);
  P[c] = P[c] + Pcorr[c];
}

// VelocityCorrection (fluid.F90:210-224): the velocity update; C1: cRK == 1,
// whose products are identities
template <bool UNIT, bool C1>
__global__ void k_velocity_correction(Geom g, double* u, double* v, double* w, const double* P, const double* Px,
                                      const double* Py, const double* Pz, double cRK) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint32_t)g.nint) return;
  int i, j, k;
  interior_ijk(g, t, i, j, k);
  const long long sj = g.ni, sk = (long long)g.ni * g.nj;
  const long long c = field_off(g, i, j, k);
  const double dt = g.dt;
  const double dPx = P[c] - P[c - 1], dPy = P[c] - P[c - sj], dPz = P[c] - P[c - sk];
  u[c] = u[c] + (C1 ? Px[c] : cRK * Px[c]) * dt - div_split(by_h<UNIT>(C1 ? dPx : cRK * dPx, g.h[0]) * dt, g.srhof);
  v[c] = v[c] + (C1 ? Py[c] : cRK * Py[c]) * dt - div_split(by_h<UNIT>(C1 ? dPy : cRK * dPy, g.h[1]) * dt, g.srhof);
  w[c] = w[c] + (C1 ? Pz[c] : cRK * Pz[c]) * dt - div_split(by_h<UNIT>(C1 ? dPz : cRK * dPz, g.h[2]) * dt, g.srhof);
}

// the vorticity of the corrected field (fluid.F90:225-234)
template <bool UNIT>
__global__ void k_vorticity(Geom g, const double* u, const double* v, const double* w, double* ox, double* oy,
                            double* oz) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint32_t)g.nint) return;
  int i, j, k;
  interior_ijk(g, t, i, j, k);
  const long long sj = g.ni, sk = (long long)g.ni * g.nj;
  const long long c = field_off(g, i, j, k);
  ox[c] = by_h<UNIT>(w[c + sj] - w[c], g.h[1]) - by_h<UNIT>(v[c + sk] - v[c], g.h[2]);
  oy[c] = by_h<UNIT>(u[c + sk] - u[c], g.h[2]) - by_h<UNIT>(w[c + 1] - w[c], g.h[0]);
  oz[c] = by_h<UNIT>(v[c + 1] - v[c], g.h[0]) - by_h<UNIT>(u[c + sj] - u[c], g.h[1]);
}

// ModifyBulkVelocity (fluid.F90:155-195): block b sums the interior nodes
// [b*per, (b+1)*per) in node order, one running sum per component
__global__ void k_bulk_partial(Geom g, const double* u, const double* v, const double* w, double* part, int per) {
  __shared__ double sh[3][kFBlock];
  const long long t0 = (long long)blockIdx.x * per;
  const long long t1 = std::min<long long>(t0 + per, g.nint);
  // thread r sums the nodes r, r + kFBlock, ... of the block's range (warps
  // read consecutive nodes), then threads 0..2 add the 256 sums in order
  double su = 0.0, sv = 0.0, sw = 0.0;
  for (long long t = t0 + threadIdx.x; t < t1; t += kFBlock) {
    int i, j, k;
    interior_ijk(g, (uint32_t)t, i, j, k);
    const long long c = field_off(g, i, j, k);
    su = su + u[c];
    sv = sv + v[c];
    sw = sw + w[c];
  }
  sh[0][threadIdx.x] = su;
  sh[1][threadIdx.x] = sv;
  sh[2][threadIdx.x] = sw;
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int r = 0; r < kFBlock; ++r) s = s + sh[threadIdx.x][r];
    part[3 * blockIdx.x + threadIdx.x] = s;
  }
}

// the blocks' sums in order, then modifyP (fluid.F90:179-185)
__global__ void k_bulk_modify(Geom g, const double* part, int nblk, double* modify, int swU, int swV, int swW,
                              double bulkU, double bulkV, double bulkW) {
  if (threadIdx.x >= 3) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s = s + part[3 * b + threadIdx.x];
  const int sw = threadIdx.x == 0 ? swU : (threadIdx.x == 1 ? swV : swW);
  const double bulk = threadIdx.x == 0 ? bulkU : (threadIdx.x == 1 ? bulkV : bulkW);
  const double nTot = (double)((long long)g.n[0] * g.n[1] * g.n[2]);
  modify[threadIdx.x] = sw == 1 ? -(s / nTot - bulk) / g.dt : 0.0;
}

__global__ void k_bulk_apply(Geom g, double* u, double* v, double* w, const double* modify) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint32_t)g.nint) return;
  int i, j, k;
  interior_ijk(g, t, i, j, k);
  const long long c = field_off(g, i, j, k);
  const double dt = g.dt;
  u[c] = u[c] + dt * modify[0];
  v[c] = v[c] + dt * modify[1];
  w[c] = w[c] + dt * modify[2];
}

// FillGhostRegionForFluid (boundary.F90:122-147), one face: the send box
// (interior layers next to `from`, earlier axes with their halo) copied into
// the halo beyond face `recv`, mirrored about a wall with u,v,w negated
struct FaceCopy {
  int lo[3], hi[3];  // send box (1-based, inclusive)
  int d;             // axis of the face
  int rlo, rinc;     // receive layer of send layer t along d: rlo + t*rinc
  int nr;            // receive layers
  int wall;
};
struct CarriedFields {
  double* f[6];  // u, v, w, P, omegaZ, Pcorr
};

__global__ void k_fill_face(Geom g, FaceCopy fc, CarriedFields cf) {
  const int ext[3] = {fc.hi[0] - fc.lo[0] + 1, fc.hi[1] - fc.lo[1] + 1, fc.hi[2] - fc.lo[2] + 1};
  const long long n = (long long)ext[0] * ext[1] * ext[2];
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int src[3];
  src[0] = fc.lo[0] + (int)(q % ext[0]);
  src[1] = fc.lo[1] + (int)((q / ext[0]) % ext[1]);
  src[2] = fc.lo[2] + (int)(q / ((long long)ext[0] * ext[1]));
  const int tl = src[fc.d] - fc.lo[fc.d];
  if (tl >= fc.nr) return;
  int dst[3] = {src[0], src[1], src[2]};
  dst[fc.d] = fc.rlo + tl * fc.rinc;
  const long long a = field_off(g, dst[0], dst[1], dst[2]), s = field_off(g, src[0], src[1], src[2]);
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const double x = cf.f[f][s];
    cf.f[f][a] = (fc.wall && f < 3) ? -x : x;
  }
}

// Boundary (fluid.F90:240-249), one walled side: the wall-normal component
// on the face layer and beyond it
__global__ void k_boundary_side(Geom g, double* f, int d, int lo_d, int hi_d) {
  int ext[3] = {g.ni, g.nj, g.nk};
  ext[d] = hi_d - lo_d + 1;
  const long long n = (long long)ext[0] * ext[1] * ext[2];
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int p[3];
  p[0] = (int)(q % ext[0]);
  p[1] = (int)((q / ext[0]) % ext[1]);
  p[2] = (int)(q / ((long long)ext[0] * ext[1]));
  for (int e = 0; e < 3; ++e) p[e] += (e == d ? lo_d : -1);  // other axes from lg = -1
  f[field_off(g, p[0], p[1], p[2])] = 0.0;
}

unsigned interior_blocks(const Ctx& c) { return (unsigned)((c.g.nint + kFBlock - 1) / kFBlock); }

}  // namespace

// the fields of the fluid stencils beyond the particle side's, on first use
static int fluid_alloc(Ctx& c) {
  if (c.ffield[IBMDEM_FLUID_UOLD]) return IBMDEM_OK;
  const size_t n = std::max<size_t>((size_t)c.g.ncell, 1);
  for (int q = IBMDEM_FLUID_UOLD; q < IBMDEM_FLUID_NFIELDS; ++q) {
    if (cudaMallocAsync(reinterpret_cast<void**>(&c.ffield[q]), n * sizeof(double), c.stream) != cudaSuccess)
      return IBMDEM_ENOMEM;
    cudaMemsetAsync(c.ffield[q], 0, n * sizeof(double), c.stream);
    c.bytes += n * sizeof(double);
  }
  if (cudaMallocAsync(reinterpret_cast<void**>(&c.fnew), 3 * n * sizeof(double), c.stream) != cudaSuccess)
    return IBMDEM_ENOMEM;
  if (cudaMallocAsync(reinterpret_cast<void**>(&c.fsum), (3 * kSumBlocks + 3) * sizeof(double), c.stream) !=
      cudaSuccess)
    return IBMDEM_ENOMEM;
  c.bytes += (3 * n + 3 * kSumBlocks + 3) * sizeof(double);
  return IBMDEM_OK;
}

int fluid_fields(Ctx& c) { return fluid_alloc(c); }

void fluid_release(Ctx& c) {
  for (int q = IBMDEM_FLUID_UOLD; q < IBMDEM_FLUID_NFIELDS; ++q)
    if (c.ffield[q]) cudaFreeAsync(c.ffield[q], c.stream);
  if (c.fnew) cudaFreeAsync(c.fnew, c.stream);
  if (c.fsum) cudaFreeAsync(c.fsum, c.stream);
  for (auto& p : c.ffield) p = nullptr;
  c.fnew = c.fsum = nullptr;
}

static double* fluid_field(Ctx& c, int which) {
  switch (which) {
    case IBMDEM_FLUID_U: return c.u;
    case IBMDEM_FLUID_V: return c.v;
    case IBMDEM_FLUID_W: return c.w;
    case IBMDEM_FLUID_FX: return c.fx;
    case IBMDEM_FLUID_FY: return c.fy;
    case IBMDEM_FLUID_FZ: return c.fz;
    default: return (which > IBMDEM_FLUID_FZ && which < IBMDEM_FLUID_NFIELDS) ? c.ffield[which] : nullptr;
  }
}

}  // namespace ibmdem

using namespace ibmdem;

// entry points: argument and state checks, then the launches on the context's stream
static int fluid_enter(ibmdem_ctx* h, const char* fn) {
  if (!h) return IBMDEM_EINVAL;
  Ctx& c = h->c;
  if (cudaSetDevice(c.device) != cudaSuccess) return IBMDEM_ECUDA;
  if (!c.haveFluid) {
    c.err = std::string(fn) + ": no fluid field (ibmdem_set_fluid first)";
    return IBMDEM_ESTATE;
  }
  wait_fields_read(c);
  if (fluid_alloc(c) != IBMDEM_OK) {
    c.err = std::string(fn) + ": out of device memory for the fluid fields";
    return IBMDEM_ENOMEM;
  }
  return IBMDEM_OK;
}

static int fluid_launched(ibmdem_ctx* h, const char* fn) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->c.err = std::string(fn) + ": " + cudaGetErrorString(e);
    return IBMDEM_ECUDA;
  }
  return IBMDEM_OK;
}

int ibmdem_set_fluid_params(ibmdem_ctx* h, double visc, double CPx, double CPy, double CPz) {
  if (!h) return IBMDEM_EINVAL;
  h->c.visc = visc;
  h->c.CPx = CPx;
  h->c.CPy = CPy;
  h->c.CPz = CPz;
  return IBMDEM_OK;
}

int ibmdem_set_fluid_field(ibmdem_ctx* h, int32_t which, const double* a) {
  int rc = fluid_enter(h, "ibmdem_set_fluid_field");
  if (rc) return rc;
  Ctx& c = h->c;
  double* d = fluid_field(c, which);
  if (!d || !a) {
    c.err = "ibmdem_set_fluid_field: bad field or null array";
    return IBMDEM_EINVAL;
  }
  c.compDoneAt = -1;  // the fields change after the last forcing loop
  if (cudaMemcpyAsync(d, a, sizeof(double) * (size_t)c.g.ncell, cudaMemcpyHostToDevice, c.stream) != cudaSuccess ||
      cudaStreamSynchronize(c.stream) != cudaSuccess)
    return IBMDEM_ECUDA;
  return IBMDEM_OK;
}

int ibmdem_get_fluid_field(ibmdem_ctx* h, int32_t which, double* a) {
  int rc = fluid_enter(h, "ibmdem_get_fluid_field");
  if (rc) return rc;
  Ctx& c = h->c;
  double* d = fluid_field(c, which);
  if (!d || !a) {
    c.err = "ibmdem_get_fluid_field: bad field or null array";
    return IBMDEM_EINVAL;
  }
  if (cudaMemcpyAsync(a, d, sizeof(double) * (size_t)c.g.ncell, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess ||
      cudaStreamSynchronize(c.stream) != cudaSuccess)
    return IBMDEM_ECUDA;
  return IBMDEM_OK;
}

int ibmdem_StoreOldVelocity(ibmdem_ctx* h) {
  int rc = fluid_enter(h, "ibmdem_StoreOldVelocity");
  if (rc) return rc;
  Ctx& c = h->c;
  const size_t nb = sizeof(double) * (size_t)c.g.ncell;
  cudaMemcpyAsync(c.ffield[IBMDEM_FLUID_UOLD], c.u, nb, cudaMemcpyDeviceToDevice, c.stream);
  cudaMemcpyAsync(c.ffield[IBMDEM_FLUID_VOLD], c.v, nb, cudaMemcpyDeviceToDevice, c.stream);
  cudaMemcpyAsync(c.ffield[IBMDEM_FLUID_WOLD], c.w, nb, cudaMemcpyDeviceToDevice, c.stream);
  return fluid_launched(h, "ibmdem_StoreOldVelocity");
}

int ibmdem_VelocityGuess(ibmdem_ctx* h, double aRK, double bRK, double cRK) {
  int rc = fluid_enter(h, "ibmdem_VelocityGuess");
  if (rc) return rc;
  Ctx& c = h->c;
  const size_t n = (size_t)c.g.ncell;
  FluidPtrs f;
  f.u = c.u;
  f.v = c.v;
  f.w = c.w;
  f.P = c.ffield[IBMDEM_FLUID_P];
  f.fx = c.fx;
  f.fy = c.fy;
  f.fz = c.fz;
  f.uold = c.ffield[IBMDEM_FLUID_UOLD];
  f.vold = c.ffield[IBMDEM_FLUID_VOLD];
  f.wold = c.ffield[IBMDEM_FLUID_WOLD];
  f.nu = c.fnew;
  f.nv = c.fnew + n;
  f.nw = c.fnew + 2 * n;
  f.Px = c.ffield[IBMDEM_FLUID_PX];
  f.Py = c.ffield[IBMDEM_FLUID_PY];
  f.Pz = c.ffield[IBMDEM_FLUID_PZ];
  f.RHSul = c.ffield[IBMDEM_FLUID_RHSUL];
  f.RHSvl = c.ffield[IBMDEM_FLUID_RHSVL];
  f.RHSwl = c.ffield[IBMDEM_FLUID_RHSWL];
  const unsigned nb = interior_blocks(c);
  PhaseScope ps(c, P_FGUESS);
  const int variant = (c.g.unit_h ? 4 : 0) | (aRK == 1.0 ? 2 : 0) | (cRK == 1.0 ? 1 : 0);
  decltype(&k_velocity_guess<true, true, true>) kern[8] = {
      k_velocity_guess<false, false, false>, k_velocity_guess<false, false, true>,
      k_velocity_guess<false, true, false>,  k_velocity_guess<false, true, true>,
      k_velocity_guess<true, false, false>,  k_velocity_guess<true, false, true>,
      k_velocity_guess<true, true, false>,   k_velocity_guess<true, true, true>};
  kern[variant]<<<nb, kFBlock, 0, c.stream>>>(c.g, f, aRK, bRK, cRK, c.visc, c.CPx, c.CPy, c.CPz);
  k_copy_interior3<<<nb, kFBlock, 0, c.stream>>>(c.g, f.nu, f.nv, f.nw, c.u, c.v, c.w);
  c.launches += 2;
  return fluid_launched(h, "ibmdem_VelocityGuess");
}

int ibmdem_FillGhostRegionForFluid(ibmdem_ctx* h) {
  int rc = fluid_enter(h, "ibmdem_FillGhostRegionForFluid");
  if (rc) return rc;
  Ctx& c = h->c;
  const Geom& g = c.g;
  CarriedFields cf{{c.u, c.v, c.w, c.ffield[IBMDEM_FLUID_P], c.ffield[IBMDEM_FLUID_OMEGAZ],
                    c.ffield[IBMDEM_FLUID_PCORR]}};
  const int SG = 1, H = 2;
  PhaseScope ps(c, P_FHALO);
  for (int s = 0; s < 6; ++s) {
    const int sideSend = s, sideRecv = (s % 2 == 0) ? s + 1 : s - 1;
    const int d = sideRecv / 2;
    const int wall = g.wall[d];
    const int from = wall ? sideRecv : sideSend;  // DealWithBoundaryFluid reads sendIdxFluid(:,sideRecv)
    FaceCopy fc;
    for (int e = 0; e < 3; ++e) {
      fc.lo[e] = e < d ? SG - H : SG;
      fc.hi[e] = e < d ? g.n[e] + H : g.n[e];
    }
    const int n = g.n[d];
    const bool fromHigh = from % 2 == 1, recvHigh = sideRecv % 2 == 1;
    fc.lo[d] = fromHigh ? n - H + 1 : SG;
    fc.hi[d] = fromHigh ? n : SG + H - 1;
    fc.d = d;
    fc.wall = wall;
    if (!wall) {
      fc.rlo = recvHigh ? n + 1 : SG - H;
      fc.rinc = 1;
    } else {  // walls fill outward from the face
      fc.rlo = recvHigh ? n + H : SG - 1;
      fc.rinc = -1;
    }
    fc.nr = H;
    const long long cells = (long long)(fc.hi[0] - fc.lo[0] + 1) * (fc.hi[1] - fc.lo[1] + 1) * (fc.hi[2] - fc.lo[2] + 1);
    k_fill_face<<<(unsigned)((cells + kFBlock - 1) / kFBlock), kFBlock, 0, c.stream>>>(g, fc, cf);
    c.launches++;
  }
  return fluid_launched(h, "ibmdem_FillGhostRegionForFluid");
}

int ibmdem_Boundary(ibmdem_ctx* h) {
  int rc = fluid_enter(h, "ibmdem_Boundary");
  if (rc) return rc;
  Ctx& c = h->c;
  const Geom& g = c.g;
  double* comp[3] = {c.u, c.v, c.w};
  PhaseScope ps(c, P_FHALO);
  for (int side = 0; side < 6; ++side) {
    const int d = side / 2;
    if (!g.wall[d]) continue;
    const int lo = side % 2 == 0 ? -1 : g.n[d] + 1;  // lg..sg or eg+1..ug
    const int hi = side % 2 == 0 ? 1 : g.n[d] + 2;
    int ext[3] = {g.ni, g.nj, g.nk};
    ext[d] = hi - lo + 1;
    const long long cells = (long long)ext[0] * ext[1] * ext[2];
    k_boundary_side<<<(unsigned)((cells + kFBlock - 1) / kFBlock), kFBlock, 0, c.stream>>>(g, comp[d], d, lo, hi);
    c.launches++;
  }
  return fluid_launched(h, "ibmdem_Boundary");
}

int ibmdem_ModifyBulkVelocity(ibmdem_ctx* h, int32_t swU, int32_t swV, int32_t swW, double bulkU, double bulkV,
                              double bulkW) {
  if (!(swU == 1 || swV == 1 || swW == 1)) return h ? IBMDEM_OK : IBMDEM_EINVAL;
  int rc = fluid_enter(h, "ibmdem_ModifyBulkVelocity");
  if (rc) return rc;
  Ctx& c = h->c;
  const long long nint = c.g.nint;
  const int nblk = (int)std::min<long long>(kSumBlocks, std::max<long long>(1, (nint + kFBlock - 1) / kFBlock));
  const int per = (int)((nint + nblk - 1) / nblk);
  double* modify = c.fsum + 3 * kSumBlocks;
  PhaseScope ps(c, P_FOTHER);
  k_bulk_partial<<<nblk, kFBlock, 0, c.stream>>>(c.g, c.u, c.v, c.w, c.fsum, per);
  k_bulk_modify<<<1, 32, 0, c.stream>>>(c.g, c.fsum, nblk, modify, swU, swV, swW, bulkU, bulkV, bulkW);
  k_bulk_apply<<<interior_blocks(c), kFBlock, 0, c.stream>>>(c.g, c.u, c.v, c.w, modify);
  c.launches += 3;
  return fluid_launched(h, "ibmdem_ModifyBulkVelocity");
}

int ibmdem_VelocityDivergence(ibmdem_ctx* h, double cRK) {
  int rc = fluid_enter(h, "ibmdem_VelocityDivergence");
  if (rc) return rc;
  Ctx& c = h->c;
  const unsigned nb = interior_blocks(c);
  PhaseScope ps(c, P_FOTHER);
  if (c.g.unit_h)
    k_velocity_divergence<true><<<nb, kFBlock, 0, c.stream>>>(c.g, c.u, c.v, c.w, c.ffield[IBMDEM_FLUID_VELDIV],
                                                             split_recip(cRK));
  else
    k_velocity_divergence<false><<<nb, kFBlock, 0, c.stream>>>(c.g, c.u, c.v, c.w, c.ffield[IBMDEM_FLUID_VELDIV],
                                                              split_recip(cRK));
  c.launches++;
  return fluid_launched(h, "ibmdem_VelocityDivergence");
}

int ibmdem_PressureCorrection(ibmdem_ctx* h, const double* Pcorr) {
  int rc = fluid_enter(h, "ibmdem_PressureCorrection");
  if (rc) return rc;
  Ctx& c = h->c;
  if (Pcorr && cudaMemcpyAsync(c.ffield[IBMDEM_FLUID_PCORR], Pcorr, sizeof(double) * (size_t)c.g.ncell,
                               cudaMemcpyHostToDevice, c.stream) != cudaSuccess)
    return IBMDEM_ECUDA;
  {
    PhaseScope ps(c, P_FOTHER);
    k_pressure_correction<<<interior_blocks(c), kFBlock, 0, c.stream>>>(c.g, c.ffield[IBMDEM_FLUID_P],
                                                                          c.ffield[IBMDEM_FLUID_PCORR]);
  }
  c.launches++;
  rc = fluid_launched(h, "ibmdem_PressureCorrection");
  // the caller may reuse Pcorr when this returns
  if (!rc && Pcorr && cudaStreamSynchronize(c.stream) != cudaSuccess) return IBMDEM_ECUDA;
  return rc;
}

int ibmdem_VelocityCorrection(ibmdem_ctx* h, double cRK) {
  int rc = fluid_enter(h, "ibmdem_VelocityCorrection");
  if (rc) return rc;
  Ctx& c = h->c;
  const unsigned nb = interior_blocks(c);
  double** F = c.ffield;
  PhaseScope ps(c, P_FOTHER);
  auto corr = c.g.unit_h ? (cRK == 1.0 ? k_velocity_correction<true, true> : k_velocity_correction<true, false>)
                         : (cRK == 1.0 ? k_velocity_correction<false, true> : k_velocity_correction<false, false>);
  corr<<<nb, kFBlock, 0, c.stream>>>(c.g, c.u, c.v, c.w, F[IBMDEM_FLUID_P], F[IBMDEM_FLUID_PX], F[IBMDEM_FLUID_PY],
                                     F[IBMDEM_FLUID_PZ], cRK);
  if (c.g.unit_h) {
    k_vorticity<true><<<nb, kFBlock, 0, c.stream>>>(c.g, c.u, c.v, c.w, F[IBMDEM_FLUID_OMEGAX], F[IBMDEM_FLUID_OMEGAY],
                                                    F[IBMDEM_FLUID_OMEGAZ]);
  } else {
    k_vorticity<false><<<nb, kFBlock, 0, c.stream>>>(c.g, c.u, c.v, c.w, F[IBMDEM_FLUID_OMEGAX],
                                                     F[IBMDEM_FLUID_OMEGAY], F[IBMDEM_FLUID_OMEGAZ]);
  }
  c.launches += 2;
  return fluid_launched(h, "ibmdem_VelocityCorrection");
}
