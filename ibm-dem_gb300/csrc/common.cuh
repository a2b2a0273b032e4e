// common.cuh — shared definitions of the GB300 IBM-DEM particle hot path.
//
// Device data layout
//   parcels   structure of arrays, field-major: recD[f*cap + i] (22 doubles per
//             parcel) and recI[f*cap + i] (3 ints).  Index i is the reference's
//             part(i+1): locals first (0..npLocal), then periodic images.
//   fields    u,v,w,fx,fy,fz in the reference's Fortran layout with the 2-cell
//             halo: offset = ((k+1)*nj + (j+1))*ni + (i+1) for i in -1..nx+2.
//   weights   W[i*84 + comp*28 + kz*9 + ky*3 + kx]: the 27 non-zero delta
//             weights per component in stencil order, 28-double aligned rows.
//   plan      the spread order: (node, contribution) pairs sorted by node with
//             the reference's part order inside each node.
// All FP64 arithmetic on the parity path is compiled with -fmad=false and keeps
// the reference's operation order, so results are bit-identical to the CPU
// restatement (libm-dependent cos/sin of the body rotation excepted).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "../../include/ibmdem.h"

namespace ibmdem {

constexpr int kHalo = 2;
constexpr int kSlots = 81;  // 3 components x 27 nodes
constexpr int kWStride = 84;  // doubles of W per parcel: 3 x (27 weights + 1 pad), 32-byte aligned rows
constexpr int kBlock = 256;

// double fields of a parcel record
enum : int {
  D_X = 0, D_V = 3, D_FCOL = 6, D_FDRAG = 9, D_VGAP = 12,
  D_RADEFF = 15, D_RAD, D_RHO, D_VOL, D_M, D_WDRAG, D_WSUM, ND
};
// int fields
// I_PID: the parcel's index in the array last given to ibmdem_set_parcels (images
// carry their root's); it keys the tangential contact history
enum : int { I_GIDX = 0, I_MSIDX, I_CELL, I_PID, NI };

// device error bits (Counters::err)
enum : int {
  E_RANGE = 1,     // a parcel left the grid + halo region
  E_IMGCAP = 2,    // periodic images exceed their capacity
  E_PAIRCAP = 4,   // contact pairs exceed their capacity
  E_WINDOW = 8,    // a delta stencil needed 4 nodes on one axis
  E_MSIDX = 16,    // parcel body index out of range
  E_PARTNER = 32,  // body partner list overflow
  E_PLANCAP = 64,  // spread-plan capacity exceeded
};

// Division of a 32-bit unsigned numerator by a fixed divisor d >= 2 with one
// high multiply (Granlund and Montgomery's round-up method, "Division by
// invariant integers using multiplication", PLDI 1994): with l = ceil(log2 d)
// and m = floor(2^32 (2^l - d) / d) + 1, n / d = (t + ((n - t) >> 1)) >> (l - 1)
// where t = high 32 bits of m * n, for every n < 2^32.
struct FastDiv {
  uint32_t d = 2, m = 0, s = 0;
  FastDiv() = default;
  __host__ explicit FastDiv(uint32_t div) : d(div) {
    uint32_t l = 0;
    while ((1ull << l) < div) ++l;
    m = (uint32_t)((((1ull << 32) * ((1ull << l) - div)) / div) + 1);
    s = l - 1;
  }
  __host__ __device__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
    const uint32_t t = __umulhi(n, m);
#else
    const uint32_t t = (uint32_t)(((unsigned long long)n * m) >> 32);
#endif
    return (t + ((n - t) >> 1)) >> s;
  }
};

// A divisor b with its split reciprocal: r = RN(1/b), lo = RN(1/b - r).  x/b
// correctly rounded is then q0 = RN(x*r + RN(x*lo)) (a faithful quotient, so
// its remainder x - b*q0 is exact in one FMA) corrected by RN(q0 + rem*r)
// (Markstein's correction theorem).  ok: b and 1/b normal with exponents
// within 2^+-200; div_split takes the division outside that and for x outside
// 2^-723 <= |x| < 2^777 (or x = 0), where the remainder could leave the
// normal range.
struct SplitRecip {
  double b, r, lo;
  int ok;
  int one;  // b == 1: x/b is x
};
inline SplitRecip split_recip(double b) {
  SplitRecip s;
  s.b = b;
  s.r = 1.0 / b;
  s.lo = std::fma(-b, s.r, 1.0) / b;  // the remainder 1 - b*r is exact
  s.ok = std::isnormal(b) && std::isnormal(s.r) && std::fabs(b) < 0x1p200 && std::fabs(b) > 0x1p-200;
  s.one = b == 1.0;
  return s;
}

struct Geom {
  int n[3];
  int ni, nj, nk;
  long long ncell;  // ni*nj*nk
  long long nint;   // nx*ny*nz
  double h[3];      // dx, dy, dz
  double start[3], end[3], len[3];
  double halfLen[3];  // 0.5*len (exact)
  double halfh[3];  // 0.5*di etc. (GetWeight)
  double err[3];    // di*1e-20 (AdjustParcelPosition)
  double hprod;     // dx*dy*dz
  int unit_h;       // dx == dy == dz == 1: /h, *dx*dy*dz are exact identities
  int wall[3];      // 1: the axis is bounded by two solid walls (bType 1), 0: periodic
  int anyWall;
  double dt, dtDEM, rhof, eta, cut2, knCoeff, di;
  double rdt, rdtLo; // RN(1/dt) and RN(1/dt - rdt), for div_dt
  SplitRecip sdt, srhof;  // dt and rhof as divisors (div_split)
  int divDt;         // dt and 1/dt normal with exponents within 2^+-200: div_dt may skip the division
  double g[3];
  FastDiv fdNint, fdN0, fdN1;  // interior nodes per component, nx, ny
  FastDiv fdNi, fdNj;          // nx + 4, ny + 4 (cells with the halo)
};

// image shift codes (imgShift): 2 bits per axis, and this bit for an image
// made across a solid wall (pType 1: never a contact partner)
constexpr int kWallImgBit = 6;

struct Counters {
  int npLocal, np, nImg, nActive, nPairs, nRuns, nContrib, nLast;
  int err, errInfo;
  int compStart[4];  // first run of each velocity component (and nRuns) in the spread plan
  int histSide;      // side of the tangential history the last contact-force call wrote
  int pad;
};

struct Recs {
  double* d;
  int* i;
  int cap;
  __host__ __device__ double& D(int f, int idx) const { return d[(size_t)f * cap + idx]; }
  __host__ __device__ int& I(int f, int idx) const { return i[(size_t)f * cap + idx]; }
};

// ---- index helpers -------------------------------------------------------
#ifdef __CUDACC__
// x / s.b, correctly rounded (SplitRecip)
__device__ inline double div_split(double x, const SplitRecip& s) {
  if (s.one) return x;
  const int ex = (int)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff;
  if (s.ok && (__double_as_longlong(x) << 1) == 0) return x * s.r;  // +-0 / b: a zero of the quotient's sign
  if (!s.ok || ex < 300 || ex > 1800) return x / s.b;
  const double q0 = __fma_rn(x, s.r, __dmul_rn(x, s.lo));
  const double rem = __fma_rn(-q0, s.b, x);
  return __fma_rn(rem, s.r, q0);
}
#endif

__host__ __device__ inline long long field_off(const Geom& g, int i, int j, int k) {
  return ((long long)(k + 1) * g.nj + (j + 1)) * g.ni + (i + 1);
}
// map3Dto1D (ZJS_INIT_DEM.F90:286), 1-based
__host__ __device__ inline int cell_id(const Geom& g, int i, int j, int k) {
  return (int)(field_off(g, i, j, k) + 1);
}
__host__ __device__ inline void cell_coords(const Geom& g, int id, int& i, int& j, int& k) {
  const uint32_t t = (uint32_t)(id - 1);
  const uint32_t a = g.fdNi.div(t);
  const uint32_t b = g.fdNj.div(a);
  i = (int)(t - a * (uint32_t)g.ni) - 1;
  j = (int)(a - b * (uint32_t)g.nj) - 1;
  k = (int)b - 1;
}
// floor((x-xStart)/di)+SG (ZJS_UPDATE_LIST_DEM.F90:41-43)
__device__ inline int cell_of(const Geom& g, int d, double x) {
  // (x - start) / h; with unit spacing the division by 1.0 is an identity
  const double t = x - g.start[d];
  return (int)floor(g.unit_h ? t : t / g.h[d]) + 1;
}
__device__ inline bool interior(const Geom& g, int i, int j, int k) {
  return i >= 1 && i <= g.n[0] && j >= 1 && j <= g.n[1] && k >= 1 && k <= g.n[2];
}
__device__ inline void set_err(Counters* c, int bit, int info) {
  atomicOr(&c->err, bit);
  atomicExch(&c->errInfo, info);
}
// periodic image of the body centre nearest to a marker coordinate
__device__ inline double body_ref(const Geom& g, int d, double xm, double X) {
  double L = g.len[d];
  double diff = xm - X;
  if (diff > g.halfLen[d]) return X + L;
  if (diff < -g.halfLen[d]) return X - L;
  return X;
}

// launch helpers
inline int nblocks(long long n, int bs = kBlock) { return (int)((n + bs - 1) / bs); }
// grid for a grid-stride loop over up to n items: at most 16 blocks per SM
inline int gs_blocks(long long n, int bs = kBlock) {
  long long b = (n + bs - 1) / bs;
  return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}
#define GRID_STRIDE(i, n) \
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)

}  // namespace ibmdem
