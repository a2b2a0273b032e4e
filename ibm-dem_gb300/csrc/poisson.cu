// poisson.cu — the pressure-correction Poisson solve (poisson.F90) on the
// context's device fields.
//
// The reference assembles (SetPressureCorrectionJacobian, poisson.F90:50-108)
// the 7-point operator A with A(c,c) = sum of 1/dl^2 over the neighbours that
// exist and A(c,n) = -1/dl^2 (periodic neighbours wrap, a neighbour behind a
// wall of bType 1 is absent), replaces the row of global cell 0 -- interior
// node (1,1,1) -- by the identity, sets that entry of the right-hand side to 0
// (SetPressureVector, poisson.F90:110-131) and solves A p = velDiv with PETSc
// (PoissonSolver, poisson.F90:143-155; GMRES + hypre, relative tolerance 1e-10
// in run.sh).  The solution is unique, so any solver that reaches the
// tolerance returns the same field; this one is direct:
//
//  * Every row but the pinned one says (L p)_c = b_c with L the singular
//    periodic/Neumann Laplacian.  The rows of L sum to zero over the grid, so
//    (L p)_0 = -sum_{c != 0} b_c; with that value b~_0 in the pinned row the
//    system L q = b~ is consistent, its zero-mean solution q is found by FFT,
//    and p = q - q_0 satisfies every row of A (p_0 = 0).
//  * A walled axis of n cells is the even extension of length 2n of a periodic
//    one (the mirror image of the first cell stands in for the absent
//    neighbour), so every axis is periodic on the extended grid and L is
//    diagonal in Fourier space: lambda = sum_d 4 sin^2(pi k_d / n'_d) / dl_d^2.
//
// The FFTs are FP64 and hand-written: a block holds L lines of one axis in
// shared memory and transforms them in place (radix-4 Cooley-Tukey for
// power-of-two lengths, a direct DFT otherwise), so each pass streams the
// complex grid once.  The data are real, so two rows share one complex x
// transform and only the n'/2 + 1 x columns of the half spectrum are kept and
// transformed along y and z: half the work and half the grid.  The z pass does forward transform, division by lambda and
// inverse transform while the lines are in shared memory.  Launches, on the
// context's stream: the ordered right-hand-side sum (2), x forward, y forward,
// z solve, y inverse, q_0 (1 block), x inverse writing Pcorr.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace ibmdem {

namespace {

constexpr int kPBlock = 256;
constexpr int kPSumBlocks = 1024;          // blocks of the ordered right-hand-side sum
constexpr int kMaxDirect = 2048;           // longest non-power-of-two line (direct DFT)
constexpr size_t kMaxSmem = 160 * 1024;    // dynamic shared memory of one block

struct PoisArgs {
  double2* X;            // the half spectrum along x (nh columns) of the extended grid, x fastest
  const double2* tw[3];  // exp(-2 pi i j / ne[d]), j < ne[d]
  const double* lam[3];  // 4 sin^2(pi k / ne[d]) / dl^2
  double* part;          // kPSumBlocks ordered partial sums, then S, then q_0
  int ne[3];             // extended extents (n, or 2n for a walled axis)
  int logn[3];           // log2(ne[d]) for a power of two, else -1
  int L[3];              // lines per block of each axis (x: pairs of rows)
  int nh;                // x columns kept: ne[0]/2 + 1 (the rest follow by conjugate symmetry)
  double scale;          // 1 / (ne0 ne1 ne2)
};

__device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(__fma_rn(a.x, b.x, -(a.y * b.y)), __fma_rn(a.x, b.y, a.y * b.x));
}

// one radix-4 group of 4 points (see lines_dft): the inputs with their
// twiddles applied, then the 4-point transform stored back
struct Quad {
  int i0;
  double2 a0, t1, t2, t3;
};

__device__ inline Quad quad_load(const double2* s, int b, int N, int logN, int lm, const double2* tw, bool inv) {
  const int m = 1 << lm;
  const int l = b >> (logN - 2), t = b & ((N >> 2) - 1);
  const int o = t & (m - 1);
  Quad q;
  q.i0 = l * N + ((t >> lm) << (lm + 2)) + o;
  q.a0 = s[q.i0];
  q.t2 = s[q.i0 + m];
  q.t1 = s[q.i0 + 2 * m];
  q.t3 = s[q.i0 + 3 * m];
  if (lm > 0) {
    const int sh = logN - 2 - lm;  // W^j = tw[j << sh]
    double2 w1 = tw[o << sh], w2 = tw[(2 * o) << sh], w3 = tw[(3 * o) << sh];
    if (inv) {
      w1.y = -w1.y;
      w2.y = -w2.y;
      w3.y = -w3.y;
    }
    q.t1 = cmul(q.t1, w1);
    q.t2 = cmul(q.t2, w2);
    q.t3 = cmul(q.t3, w3);
  }
  return q;
}

__device__ inline void quad_store(double2* s, const Quad& q, int m, bool inv) {
  const double2 u0 = make_double2(q.a0.x + q.t2.x, q.a0.y + q.t2.y);
  const double2 u1 = make_double2(q.a0.x - q.t2.x, q.a0.y - q.t2.y);
  const double2 u2 = make_double2(q.t1.x + q.t3.x, q.t1.y + q.t3.y);
  const double2 u3 = make_double2(q.t1.x - q.t3.x, q.t1.y - q.t3.y);
  // forward: X1 = u1 - i u3, X3 = u1 + i u3; inverse: the signs of i swap
  const double2 ju3 = inv ? make_double2(-u3.y, u3.x) : make_double2(u3.y, -u3.x);
  s[q.i0] = make_double2(u0.x + u2.x, u0.y + u2.y);
  s[q.i0 + m] = make_double2(u1.x + ju3.x, u1.y + ju3.y);
  s[q.i0 + 2 * m] = make_double2(u0.x - u2.x, u0.y - u2.y);
  s[q.i0 + 3 * m] = make_double2(u1.x - ju3.x, u1.y - ju3.y);
}

// L lines of N points in shared memory, s[l*N + j]: the DFT of each line
// (sign -1; +1 when inv), natural order in and out.  tmp: L*N more points,
// used by the direct DFT only.
__device__ void lines_dft(double2* s, double2* tmp, int N, int logN, int L, const double2* tw, bool inv) {
  if (N == 1) return;
  const int tot = L * N;
  if (logN > 0) {
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const int l = e >> logN, j = e & (N - 1);
      const int r = (int)(__brev((unsigned)j) >> (32 - logN));
      if (r > j) {
        const double2 a = s[l * N + j];
        s[l * N + j] = s[l * N + r];
        s[l * N + r] = a;
      }
    }
    __syncthreads();
    int lm = 0;
    if (logN & 1) {
      // an odd number of stages: one radix-2 stage of unit twiddles first
      for (int b = threadIdx.x; b < (tot >> 1); b += blockDim.x) {
        const int i0 = 2 * b;
        const double2 a = s[i0], c = s[i0 + 1];
        s[i0] = make_double2(a.x + c.x, a.y + c.y);
        s[i0 + 1] = make_double2(a.x - c.x, a.y - c.y);
      }
      __syncthreads();
      lm = 1;
    }
    // radix-4 stages: two radix-2 stages at once.  After the bit reversal the
    // four blocks of m points of a group of 4m hold the sub-transforms of the
    // residues 0, 2, 1, 3 (mod 4); with W = exp(-+2 pi i / 4m) the group's
    // outputs are the 4-point transform of (a0, W^o a2, W^2o a1, W^3o a3):
    // 3 complex products and 16 adds for 4 points (radix-2: 4 and 16).
    // two groups per thread and pass, both loaded before either is stored:
    // the groups are disjoint, and the second's loads overlap the first's
    // arithmetic
    const int nq = tot >> 2, bd = blockDim.x;
    for (; lm < logN; lm += 2) {
      const int m = 1 << lm;
      for (int b = threadIdx.x; b < nq; b += 2 * bd) {
        const Quad qa = quad_load(s, b, N, logN, lm, tw, inv);
        if (b + bd < nq) {
          const Quad qb = quad_load(s, b + bd, N, logN, lm, tw, inv);
          quad_store(s, qa, m, inv);
          quad_store(s, qb, m, inv);
        } else {
          quad_store(s, qa, m, inv);
        }
      }
      __syncthreads();
    }
  } else {
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const int l = e / N, k = e - l * N;
      const double2* in = s + l * N;
      double2 acc = make_double2(0.0, 0.0);
      int jk = 0;  // j*k mod N
      for (int j = 0; j < N; ++j) {
        double2 w = tw[jk];
        if (inv) w.y = -w.y;
        const double2 p = cmul(in[j], w);
        acc.x += p.x;
        acc.y += p.y;
        jk += k;
        if (jk >= N) jk -= N;
      }
      tmp[e] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < tot; e += blockDim.x) s[e] = tmp[e];
    __syncthreads();
  }
}

// position on the extended axis -> interior index (0-based) of its source node
__device__ inline int src_of(int xe, int n) { return xe < n ? xe : 2 * n - 1 - xe; }

// block b sums the right-hand side over interior nodes [b*per, (b+1)*per) in
// node order, without node 0 (the pinned row)
__global__ void k_pois_partial(Geom g, const double* b, double* part, long long per) {
  __shared__ double sh[kPBlock];
  const long long t0 = (long long)blockIdx.x * per;
  const long long t1 = std::min<long long>(t0 + per, g.nint);
  double s = 0.0;
  for (long long t = t0 + threadIdx.x; t < t1; t += kPBlock) {
    if (t == 0) continue;
    const uint32_t row = g.fdN0.div((uint32_t)t);
    const uint32_t kk = g.fdN1.div(row);
    const int i = (int)(t - row * (uint32_t)g.n[0]) + 1;
    const int j = (int)(row - kk * (uint32_t)g.n[1]) + 1;
    s = s + b[field_off(g, i, j, (int)kk + 1)];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int r = 0; r < kPBlock; ++r) a = a + sh[r];
    part[blockIdx.x] = a;
  }
}

// S = the blocks' sums in a fixed order (lane l adds blocks 32l..32l+31 in
// order, then lane 0 adds the 32 lane sums in order); the pinned row's value
// is -S.  One warp.
__global__ void k_pois_total(double* part) {
  static_assert(kPSumBlocks == 32 * 32, "one warp of 32 chunks");
  __shared__ double sh[32];
  const int l = threadIdx.x;
  double s = 0.0;
  for (int r = 0; r < 32; ++r) s = s + part[32 * l + r];
  sh[l] = s;
  __syncwarp();
  if (l == 0) {
    double t = 0.0;
    for (int r = 0; r < 32; ++r) t = t + sh[r];
    part[kPSumBlocks] = t;
  }
}

// x forward: a block holds L[0] pairs of rows (y', z') of the extended grid,
// read from the right-hand side with the mirrors of walled axes and the
// pinned value.  Rows 2p and 2p+1 are the real and imaginary parts of one
// complex line; after its transform Z, the rows' spectra are
// A(k) = (Z(k) + conj Z(N-k))/2 and B(k) = (Z(k) - conj Z(N-k))/(2i), of which
// k = 0..N/2 are kept.
__global__ void __launch_bounds__(kPBlock) k_pois_xfwd(Geom g, PoisArgs a, const double* b) {
  extern __shared__ double2 sm[];
  const int N = a.ne[0], L = a.L[0], nh = a.nh;
  double2* s = sm;
  double2* tmp = sm + L * N;
  const long long rows = (long long)a.ne[1] * a.ne[2];
  const long long r0 = 2LL * blockIdx.x * L;
  const double pinned = -a.part[kPSumBlocks];
  for (int e = threadIdx.x; e < L * N; e += blockDim.x) {
    const int l = e / N, xe = e - l * N;
    const int x = src_of(xe, g.n[0]);
    double v[2] = {0.0, 0.0};
    for (int h = 0; h < 2; ++h) {
      const long long r = r0 + 2 * l + h;
      if (r < rows) {
        const int ye = (int)(r % a.ne[1]), ze = (int)(r / a.ne[1]);
        const int y = src_of(ye, g.n[1]), z = src_of(ze, g.n[2]);
        v[h] = (x | y | z) == 0 ? pinned : b[field_off(g, x + 1, y + 1, z + 1)];
      }
    }
    s[e] = make_double2(v[0], v[1]);
  }
  __syncthreads();
  lines_dft(s, tmp, N, a.logn[0], L, a.tw[0], false);
  for (int e = threadIdx.x; e < L * nh; e += blockDim.x) {
    const int l = e / nh, k = e - l * nh;
    const long long ra = r0 + 2 * l;
    if (ra >= rows) continue;
    const double2 z = s[l * N + k];
    const double2 m = s[l * N + (k == 0 ? 0 : N - k)];  // conj(m) = conj Z(N-k)
    a.X[ra * nh + k] = make_double2(0.5 * (z.x + m.x), 0.5 * (z.y - m.y));
    if (ra + 1 < rows) a.X[(ra + 1) * nh + k] = make_double2(0.5 * (z.y + m.y), -0.5 * (z.x - m.x));
  }
}

// y or z lines (axis d = 1, 2), L[d] neighbouring x' per block so that each
// point of a line is a run of L[d] consecutive complex values.  mode 0:
// forward; 1: inverse; 2 (z only): forward, divide by lambda, inverse.
// outer: extent of the remaining axis that is transformed (z' for d = 1,
// y' for d = 2).
__global__ void __launch_bounds__(kPBlock) k_pois_lines(PoisArgs a, int d, int mode, int outer) {
  extern __shared__ double2 sm[];
  // the axis's values by selection (indexing the parameter arrays with d
  // would copy them to local memory)
  const bool y = d == 1;
  const int N = y ? a.ne[1] : a.ne[2], L = y ? a.L[1] : a.L[2], logN = y ? a.logn[1] : a.logn[2];
  const double2* tw = y ? a.tw[1] : a.tw[2];
  const int ne0 = a.nh;  // x columns of the half spectrum
  double2* s = sm;
  double2* tmp = sm + L * N;
  const int groups = (ne0 + L - 1) / L;
  const int grp = (int)(blockIdx.x % groups), o = (int)(blockIdx.x / groups);
  if (o >= outer) return;
  const int x0 = grp * L;
  const int La = min(L, ne0 - x0);  // the last group holds the columns that are left (nh is odd)
  const long long plane = (long long)ne0 * a.ne[1];
  const long long base = y ? (long long)o * plane + x0 : (long long)o * ne0 + x0;
  const long long stride = y ? ne0 : plane;
  for (int e = threadIdx.x; e < La * N; e += blockDim.x) {
    const int j = e / La, l = e - j * La;
    s[l * N + j] = a.X[base + j * stride + l];
  }
  __syncthreads();
  lines_dft(s, tmp, N, logN, La, tw, mode == 1);
  if (mode == 2) {
    // s[l*N + kz] holds the transform at (kx = x0 + l, ky = o, kz)
    const double ly = a.lam[1][o];
    for (int e = threadIdx.x; e < La * N; e += blockDim.x) {
      const int l = e / N, kz = e - l * N;
      const double den = a.lam[0][x0 + l] + ly + a.lam[2][kz];
      const double f = den > 0.0 ? a.scale / den : 0.0;
      s[e] = make_double2(s[e].x * f, s[e].y * f);
    }
    __syncthreads();
    lines_dft(s, tmp, N, logN, La, tw, true);
  }
  for (int e = threadIdx.x; e < La * N; e += blockDim.x) {
    const int j = e / La, l = e - j * La;
    a.X[base + j * stride + l] = s[l * N + j];
  }
}

// q_0 = the inverse x transform at x = 0 of row (0, 0): the real parts of
// the full spectrum summed, the conjugate half counted by doubling, in a
// fixed order (the 1/n' normalisation is in the lambda division)
__global__ void k_pois_q0(PoisArgs a) {
  if (threadIdx.x != 0) return;
  const int N = a.ne[0];
  double s = a.X[0].x, d = 0.0;
  const int last = (N & 1) ? a.nh - 1 : a.nh - 2;  // the bins with a distinct conjugate
  for (int k = 1; k <= last; ++k) d = d + a.X[k].x;
  s = s + 2.0 * d;
  if (!(N & 1) && N > 1) s = s + a.X[N / 2].x;
  a.part[kPSumBlocks + 1] = s;
}

// x inverse over pairs of rows of the original grid: Z = A + iB from the two
// rows' half spectra (the other half by conjugate symmetry), one complex
// inverse transform, the rows in its real and imaginary parts; Pcorr = q - q_0
// (exactly 0 at the pinned node)
__global__ void __launch_bounds__(kPBlock) k_pois_xinv(Geom g, PoisArgs a, double* pc) {
  extern __shared__ double2 sm[];
  const int N = a.ne[0], L = a.L[0], nh = a.nh;
  double2* s = sm;
  double2* tmp = sm + L * N;
  const long long rows = (long long)g.n[1] * g.n[2];
  const long long r0 = 2LL * blockIdx.x * L;
  for (int e = threadIdx.x; e < L * N; e += blockDim.x) {
    const int l = e / N, k = e - l * N;
    const bool lo = k < nh;
    const int kk = lo ? k : N - k;
    double2 v[2];
    for (int h = 0; h < 2; ++h) {
      const long long r = r0 + 2 * l + h;
      v[h] = make_double2(0.0, 0.0);
      if (r < rows) {
        const long long y = r % g.n[1], z = r / g.n[1];
        v[h] = a.X[(z * a.ne[1] + y) * nh + kk];
        if (!lo) v[h].y = -v[h].y;
      }
    }
    s[e] = make_double2(v[0].x - v[1].y, v[0].y + v[1].x);
  }
  __syncthreads();
  lines_dft(s, tmp, N, a.logn[0], L, a.tw[0], true);
  const double q0 = a.part[kPSumBlocks + 1];
  for (int e = threadIdx.x; e < L * N; e += blockDim.x) {
    const int l = e / N, x = e - l * N;
    if (x >= g.n[0]) continue;
    for (int h = 0; h < 2; ++h) {
      const long long r = r0 + 2 * l + h;
      if (r >= rows) break;
      const int y = (int)(r % g.n[1]), z = (int)(r / g.n[1]);
      const double q = h == 0 ? s[e].x : s[e].y;
      pc[field_off(g, x + 1, y + 1, z + 1)] = (x | y | z) == 0 ? 0.0 : q - q0;
    }
  }
}

int ilog2_exact(int n) {
  if (n <= 0 || (n & (n - 1))) return -1;
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

// lines per block: as many as fit in 64 KB (direct DFT: twice the points)
int lines_per_block(int n, bool direct, int cap) {
  const size_t per = (size_t)n * sizeof(double2) * (direct ? 2 : 1);
  int L = 1;
  while (L < cap && (size_t)(2 * L) * per <= 64 * 1024) L *= 2;
  return L;
}

size_t smem_of(const PoisArgs& a, int d) {
  return (size_t)a.L[d] * a.ne[d] * sizeof(double2) * (a.logn[d] < 0 ? 2 : 1);
}

}  // namespace

// the plan of the solve on first use: extended extents, twiddles, eigenvalues
static int poisson_plan(Ctx& c) {
  PoissonPlan& p = c.pois;
  if (p.X) return IBMDEM_OK;
  size_t tot = 1, aux = kPSumBlocks + 2;
  for (int d = 0; d < 3; ++d) {
    p.ne[d] = c.g.wall[d] ? 2 * c.g.n[d] : c.g.n[d];
    p.logn[d] = ilog2_exact(p.ne[d]);
    if (p.logn[d] < 0 && p.ne[d] > kMaxDirect) {
      c.err = "ibmdem_PoissonSolver: an extended extent that is not a power of two is longer than 2048";
      return IBMDEM_EUNSUPPORTED;
    }
    if ((size_t)p.ne[d] * sizeof(double2) * (p.logn[d] < 0 ? 2 : 1) > kMaxSmem) {
      c.err = "ibmdem_PoissonSolver: a line of the extended grid does not fit in shared memory";
      return IBMDEM_EUNSUPPORTED;
    }
    tot *= (size_t)p.ne[d];
    aux += 3 * (size_t)p.ne[d];
  }
  // host tables: the twiddles from sin/cos of exact dyadic or rational angles
  std::vector<double> h(aux, 0.0);
  size_t off = 0;
  for (int d = 0; d < 3; ++d) {
    p.twOff[d] = off;
    const int n = p.ne[d];
    for (int j = 0; j < n; ++j) {
      const double ang = 2.0 * M_PI * (double)j / (double)n;
      h[off + 2 * j] = std::cos(ang);
      h[off + 2 * j + 1] = -std::sin(ang);
    }
    off += 2 * (size_t)n;
  }
  for (int d = 0; d < 3; ++d) {
    p.lamOff[d] = off;
    const int n = p.ne[d];
    const double dl2 = c.g.h[d] * c.g.h[d];
    for (int k = 0; k < n; ++k) {
      const double sn = std::sin(M_PI * (double)k / (double)n);
      h[off + k] = 4.0 * sn * sn / dl2;
    }
    off += (size_t)n;
  }
  p.partOff = off;
  p.nh = p.ne[0] / 2 + 1;
  const size_t half = (size_t)p.nh * p.ne[1] * p.ne[2];
  if (cudaMallocAsync(reinterpret_cast<void**>(&p.X), half * sizeof(double2), c.stream) != cudaSuccess) {
    p.X = nullptr;
    c.err = "ibmdem_PoissonSolver: out of device memory for the transform grid";
    return IBMDEM_ENOMEM;
  }
  if (cudaMallocAsync(reinterpret_cast<void**>(&p.aux), aux * sizeof(double), c.stream) != cudaSuccess) {
    cudaFreeAsync(p.X, c.stream);
    p.X = nullptr;
    p.aux = nullptr;
    c.err = "ibmdem_PoissonSolver: out of device memory for the transform tables";
    return IBMDEM_ENOMEM;
  }
  if (cudaMemcpyAsync(p.aux, h.data(), aux * sizeof(double), cudaMemcpyHostToDevice, c.stream) != cudaSuccess ||
      cudaStreamSynchronize(c.stream) != cudaSuccess) {
    // no half-built plan: the next call plans again
    cudaFreeAsync(p.X, c.stream);
    cudaFreeAsync(p.aux, c.stream);
    p.X = nullptr;
    p.aux = nullptr;
    c.err = "ibmdem_PoissonSolver: the transform tables could not be uploaded";
    return IBMDEM_ECUDA;
  }
  p.total = (long long)tot;
  c.bytes += half * sizeof(double2) + aux * sizeof(double);
  cudaFuncSetAttribute(k_pois_xfwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
  cudaFuncSetAttribute(k_pois_lines, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
  cudaFuncSetAttribute(k_pois_xinv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
  return IBMDEM_OK;
}

void poisson_release(Ctx& c) {
  PoissonPlan& p = c.pois;
  if (p.X) cudaFreeAsync(p.X, c.stream);
  if (p.aux) cudaFreeAsync(p.aux, c.stream);
  p.X = nullptr;
  p.aux = nullptr;
}

}  // namespace ibmdem

using namespace ibmdem;

// SetPressureVector + PoissonSolver + GetLocalArray (poisson.F90:110-186):
// Pcorr on the interior nodes from velDiv; the halo of Pcorr is left as it is
// (FillGhostRegionForFluid fills it).  The matrix (InitPressureCorrectionMatrix,
// SetPressureCorrectionJacobian, SetKSP) is the plan built on the first call.
int ibmdem_PoissonSolver(ibmdem_ctx* h) {
  if (!h) return IBMDEM_EINVAL;
  Ctx& c = h->c;
  if (cudaSetDevice(c.device) != cudaSuccess) return IBMDEM_ECUDA;
  if (!c.haveFluid) {
    c.err = "ibmdem_PoissonSolver: no fluid field (ibmdem_set_fluid first)";
    return IBMDEM_ESTATE;
  }
  wait_fields_read(c);
  if (fluid_fields(c) != IBMDEM_OK) {
    c.err = "ibmdem_PoissonSolver: out of device memory for the fluid fields";
    return IBMDEM_ENOMEM;
  }
  int rc = poisson_plan(c);
  if (rc) return rc;
  PoissonPlan& p = c.pois;
  PoisArgs a;
  a.X = p.X;
  for (int d = 0; d < 3; ++d) {
    a.tw[d] = reinterpret_cast<const double2*>(p.aux + p.twOff[d]);
    a.lam[d] = p.aux + p.lamOff[d];
    a.ne[d] = p.ne[d];
    a.logn[d] = p.logn[d];
  }
  a.part = p.aux + p.partOff;
  a.scale = 1.0 / (double)p.total;
  a.L[0] = lines_per_block(p.ne[0], p.logn[0] < 0, 8);
  a.L[1] = lines_per_block(p.ne[1], p.logn[1] < 0, 8);
  a.L[2] = lines_per_block(p.ne[2], p.logn[2] < 0, 8);
  const double* b = c.ffield[IBMDEM_FLUID_VELDIV];
  double* pc = c.ffield[IBMDEM_FLUID_PCORR];
  const long long per = (c.g.nint + kPSumBlocks - 1) / kPSumBlocks;
  a.nh = p.nh;
  const int groups = (p.nh + a.L[1] - 1) / a.L[1];
  const int groupsZ = (p.nh + a.L[2] - 1) / a.L[2];
  {
    PhaseScope ps(c, P_FPOISSON);
    k_pois_partial<<<kPSumBlocks, kPBlock, 0, c.stream>>>(c.g, b, a.part, per);
    k_pois_total<<<1, 32, 0, c.stream>>>(a.part);
    const long long rowsE = (long long)p.ne[1] * p.ne[2];
    k_pois_xfwd<<<(unsigned)((rowsE + 2 * a.L[0] - 1) / (2 * a.L[0])), kPBlock, smem_of(a, 0), c.stream>>>(c.g, a, b);
    // y forward over every z', z solve over every y', y inverse over z' < nz
    k_pois_lines<<<(unsigned)((long long)groups * p.ne[2]), kPBlock, smem_of(a, 1), c.stream>>>(a, 1, 0, p.ne[2]);
    k_pois_lines<<<(unsigned)((long long)groupsZ * p.ne[1]), kPBlock, smem_of(a, 2), c.stream>>>(a, 2, 2, p.ne[1]);
    k_pois_lines<<<(unsigned)((long long)groups * c.g.n[2]), kPBlock, smem_of(a, 1), c.stream>>>(a, 1, 1, c.g.n[2]);
    k_pois_q0<<<1, 32, 0, c.stream>>>(a);
    const long long rows = (long long)c.g.n[1] * c.g.n[2];
    k_pois_xinv<<<(unsigned)((rows + 2 * a.L[0] - 1) / (2 * a.L[0])), kPBlock, smem_of(a, 0), c.stream>>>(c.g, a, pc);
  }
  c.launches += 8;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    c.err = std::string("ibmdem_PoissonSolver: ") + cudaGetErrorString(e);
    return IBMDEM_ECUDA;
  }
  return IBMDEM_OK;
}
