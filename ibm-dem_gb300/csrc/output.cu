// output.cu — the reference's particle output files, written from device state
// without holding up the time loop.
//
// OutputCloudTecplot (ZJS_IO_DEM.F90:82-121) writes the local markers' x, v,
// MSIdx and vgap as one Tecplot point zone; the post-processing of
// fluid.F90:392-397 appends one line per body to DEM/<GlobalIdx>.probe.  Both
// use Fortran list-directed WRITE(unit,*); the lines here follow gfortran's
// list-directed layout for REAL(8) and default INTEGER items (see
// put_real / put_int) so that the files read column for column like the
// reference's.  ibmdem_output_async takes a snapshot with device-to-host copies
// on a stream of its own and formats the files on a host thread (in parallel
// chunks), so a caller's next step only waits for the copies.
#include <algorithm>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace ibmdem {

namespace {

// One REAL(8) item of list-directed output as gfortran writes it: a G25.17E3
// field.  17 significant digits, correctly rounded; with the decimal exponent
// k of the rounded value (0.1 <= |x|*10^-k < 1), 0 <= k <= 17 gives F20.(17-k)
// followed by 5 blanks, anything else 1PE25.17E3.  Zero is 0.0000000000000000.
void put_real(std::string& s, double v) {
  char buf[64];
  if (std::isnan(v) || std::isinf(v)) {
    const char* t = std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity");
    std::snprintf(buf, sizeof buf, "%25s", t);
    s += buf;
    return;
  }
  if (v == 0.0) {
    s += std::signbit(v) ? " -0.0000000000000000     " : "  0.0000000000000000     ";
    return;
  }
  char e[40];
  std::snprintf(e, sizeof e, "%.16e", v);  // [-]d.dddddddddddddddde[+-]XX
  const bool neg = e[0] == '-';
  const char* p = e + (neg ? 1 : 0);
  char digits[18];
  digits[0] = p[0];
  std::memcpy(digits + 1, p + 2, 16);
  digits[17] = 0;
  const int e10 = std::atoi(std::strchr(p, 'e') + 1);
  const int k = e10 + 1;
  std::string f;
  if (k >= 0 && k <= 17) {
    if (neg) f += '-';
    if (k == 0) {
      f += "0.";
      f += digits;
    } else {
      f.append(digits, k);
      f += '.';
      f += digits + k;
    }
    std::snprintf(buf, sizeof buf, "%20s     ", f.c_str());
  } else {
    if (neg) f += '-';
    f += digits[0];
    f += '.';
    f += digits + 1;
    char ex[16];
    std::snprintf(ex, sizeof ex, "E%c%03d", e10 < 0 ? '-' : '+', std::abs(e10));
    f += ex;
    std::snprintf(buf, sizeof buf, "%25s", f.c_str());
  }
  s += buf;
}

// One default INTEGER item: a 12-character field (I12 of gfortran's
// list-directed output for kind 4)
void put_int(std::string& s, long long v) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "%12lld", v);
  s += buf;
}

// rows of the snapshot, field-major as on the device: x[3][n], v[3][n], vgap[3][n]
struct MarkerRows {
  int n = 0;
  const double* x = nullptr;
  const double* v = nullptr;
  const double* vgap = nullptr;
  const int* msidx = nullptr;
  size_t stride = 0;  // elements between the rows of one vector
};

void marker_line(std::string& s, const MarkerRows& m, int i) {
  s += ' ';
  for (int d = 0; d < 3; ++d) put_real(s, m.x[d * m.stride + i]);
  for (int d = 0; d < 3; ++d) put_real(s, m.v[d * m.stride + i]);
  put_int(s, m.msidx[i]);
  for (int d = 0; d < 3; ++d) put_real(s, m.vgap[d * m.stride + i]);
  s += '\n';
}

int write_tecplot(const char* path, const MarkerRows& m, const double* centre) {
  std::FILE* f = std::fopen(path, "w");
  if (!f) return IBMDEM_EINVAL;
  std::string head = " variables=x,y,z,u,v,w,index,ugap,vgap,wgap\n zone i=";
  put_int(head, m.n > 0 ? m.n : 1);
  head += " j=";
  put_int(head, 1);
  head += '\n';
  bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
  if (m.n == 0) {
    // no local parcel: one point at the subdomain centre (ZJS_IO_DEM.F90:111)
    std::string s = " ";
    for (int d = 0; d < 3; ++d) put_real(s, centre[d]);
    for (int d = 0; d < 3; ++d) put_real(s, 0.0);
    put_int(s, 0);
    for (int d = 0; d < 3; ++d) put_real(s, 0.0);
    s += '\n';
    ok = ok && std::fwrite(s.data(), 1, s.size(), f) == s.size();
  } else {
    // chunks formatted in parallel, written in order
    const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int chunk = 1 << 15;
    for (int c0 = 0; c0 < m.n && ok; c0 += chunk * nt) {
      std::vector<std::string> parts(nt);
      std::vector<std::thread> th;
      for (int t = 0; t < nt; ++t) {
        const int a = c0 + t * chunk, b = std::min(m.n, a + chunk);
        if (a >= b) break;
        th.emplace_back([&, t, a, b] {
          parts[t].reserve((size_t)(b - a) * 240);
          for (int i = a; i < b; ++i) marker_line(parts[t], m, i);
        });
      }
      for (auto& x : th) x.join();
      for (auto& p : parts) ok = ok && std::fwrite(p.data(), 1, p.size(), f) == p.size();
    }
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? IBMDEM_OK : IBMDEM_EINVAL;
}

int write_probes(const char* dir, long long step, int nMS, const ibmdem_multisphere* ms, double rhof) {
  for (int b = 0; b < nMS; ++b) {
    const ibmdem_multisphere& B = ms[b];
    std::string s = " ";
    put_int(s, step);
    for (int d = 0; d < 3; ++d) put_real(s, B.x[d]);
    for (int d = 0; d < 3; ++d) put_real(s, B.v[d]);
    for (int d = 0; d < 3; ++d) put_real(s, B.omega[d]);
    for (int d = 0; d < 3; ++d) put_real(s, B.fdrag[d] / B.m * rhof);
    for (int d = 0; d < 3; ++d) put_real(s, B.fmom[d] / B.I * rhof);
    for (int d = 0; d < 3; ++d) put_real(s, B.fcol[d] / B.m);
    s += '\n';
    char name[64];
    std::snprintf(name, sizeof name, "/%d.probe", B.globalIdx);
    const std::string path = std::string(dir) + name;
    std::FILE* f = std::fopen(path.c_str(), "a");
    if (!f) return IBMDEM_EINVAL;
    const bool ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
    if (std::fclose(f) != 0 || !ok) return IBMDEM_EINVAL;
  }
  return IBMDEM_OK;
}

}  // namespace

// snapshot buffers and the writer thread of one context
struct OutputState {
  cudaStream_t copy = nullptr;
  cudaEvent_t ready = nullptr, done = nullptr;
  double* hRows = nullptr;  // [9][cap]: x, v, vgap
  int* hIdx = nullptr;      // [cap]: MSIdx
  int* hCnt = nullptr;      // npLocal at the snapshot
  ibmdem_multisphere* hBodies = nullptr;
  size_t capRows = 0;
  int capBodies = 0;
  std::thread writer;
  bool pending = false;
  int status = IBMDEM_OK;
};

void output_release(Ctx& c) {
  OutputState* o = c.out;
  if (!o) return;
  if (o->writer.joinable()) o->writer.join();
  if (o->hRows) cudaFreeHost(o->hRows);
  if (o->hIdx) cudaFreeHost(o->hIdx);
  if (o->hCnt) cudaFreeHost(o->hCnt);
  if (o->hBodies) cudaFreeHost(o->hBodies);
  if (o->ready) cudaEventDestroy(o->ready);
  if (o->done) cudaEventDestroy(o->done);
  if (o->copy) cudaStreamDestroy(o->copy);
  delete o;
  c.out = nullptr;
}

}  // namespace ibmdem

using namespace ibmdem;

extern "C" {

int ibmdem_write_tecplot_markers(const char* path, int32_t n, const ibmdem_parcel* parts, const double* centre) {
  if (!path || n < 0 || (n > 0 && !parts) || (n == 0 && !centre)) return IBMDEM_EINVAL;
  std::vector<double> rows((size_t)9 * n);
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) {
    for (int d = 0; d < 3; ++d) {
      rows[(size_t)d * n + i] = parts[i].x[d];
      rows[(size_t)(3 + d) * n + i] = parts[i].v[d];
      rows[(size_t)(6 + d) * n + i] = parts[i].vgap[d];
    }
    idx[i] = parts[i].MSIdx;
  }
  MarkerRows m;
  m.n = n;
  m.x = rows.data();
  m.v = rows.data() + (size_t)3 * n;
  m.vgap = rows.data() + (size_t)6 * n;
  m.msidx = idx.data();
  m.stride = (size_t)n;
  return write_tecplot(path, m, centre);
}

int ibmdem_write_body_probes(const char* dir, int64_t step, int32_t nMS, const ibmdem_multisphere* ms, double rhof) {
  if (!dir || nMS < 0 || (nMS > 0 && !ms)) return IBMDEM_EINVAL;
  return write_probes(dir, step, nMS, ms, rhof);
}

int ibmdem_output_wait(ibmdem_ctx* h) {
  if (!h) return IBMDEM_EINVAL;
  OutputState* o = h->c.out;
  if (!o || !o->pending) return IBMDEM_OK;
  if (o->writer.joinable()) o->writer.join();
  o->pending = false;
  return o->status;
}

int ibmdem_output_async(ibmdem_ctx* h, const char* tecplot_path, const char* probe_dir, int64_t step) {
  if (!h) return IBMDEM_EINVAL;
  Ctx& c = h->c;
  int rc = ibmdem_output_wait(h);
  if (rc) return rc;
  if (!tecplot_path && !probe_dir) return IBMDEM_OK;
  if (!c.haveParcels) {
    c.err = "ibmdem_output_async: no parcels";
    return IBMDEM_ESTATE;
  }
  if (cudaSetDevice(c.device) != cudaSuccess) return IBMDEM_ECUDA;
  if (!c.out) c.out = new OutputState();
  OutputState* o = c.out;
  auto fail = [&](const char* what, cudaError_t e) {
    c.err = std::string("ibmdem_output_async: ") + what + ": " + cudaGetErrorString(e);
    return IBMDEM_ECUDA;
  };
  cudaError_t e = cudaSuccess;
  if (!o->copy && (e = cudaStreamCreateWithFlags(&o->copy, cudaStreamNonBlocking)) != cudaSuccess)
    return fail("stream", e);
  if (!o->ready && (e = cudaEventCreateWithFlags(&o->ready, cudaEventDisableTiming)) != cudaSuccess)
    return fail("event", e);
  if (!o->done && (e = cudaEventCreateWithFlags(&o->done, cudaEventDisableTiming)) != cudaSuccess)
    return fail("event", e);
  const size_t cap = (size_t)c.capLocal;
  if (o->capRows < cap) {
    if (o->hRows) cudaFreeHost(o->hRows);
    if (o->hIdx) cudaFreeHost(o->hIdx);
    o->hRows = nullptr;
    o->hIdx = nullptr;
    o->capRows = 0;
    if ((e = cudaMallocHost(&o->hRows, sizeof(double) * 9 * cap)) != cudaSuccess) return fail("pinned rows", e);
    if ((e = cudaMallocHost(&o->hIdx, sizeof(int) * cap)) != cudaSuccess) return fail("pinned rows", e);
    o->capRows = cap;
  }
  if (!o->hCnt && (e = cudaMallocHost(&o->hCnt, sizeof(int))) != cudaSuccess) return fail("pinned count", e);
  if (o->capBodies < c.nMS) {
    if (o->hBodies) cudaFreeHost(o->hBodies);
    o->hBodies = nullptr;
    o->capBodies = 0;
    if ((e = cudaMallocHost(&o->hBodies, sizeof(ibmdem_multisphere) * c.nMS)) != cudaSuccess)
      return fail("pinned bodies", e);
    o->capBodies = c.nMS;
  }
  // copies after the work issued so far; later context work waits for them
  cudaEventRecord(o->ready, c.stream);
  cudaStreamWaitEvent(o->copy, o->ready, 0);
  const size_t rc0 = (size_t)c.cap;  // device row stride
  const double* D = c.recD[c.cur];
  const int* I = c.recI[c.cur];
  const int srcRow[9] = {D_X, D_X + 1, D_X + 2, D_V, D_V + 1, D_V + 2, D_VGAP, D_VGAP + 1, D_VGAP + 2};
  if (tecplot_path && cap > 0) {
    for (int r = 0; r < 9; ++r)
      cudaMemcpyAsync(o->hRows + (size_t)r * cap, D + (size_t)srcRow[r] * rc0, sizeof(double) * cap,
                      cudaMemcpyDeviceToHost, o->copy);
    cudaMemcpyAsync(o->hIdx, I + (size_t)I_MSIDX * rc0, sizeof(int) * cap, cudaMemcpyDeviceToHost, o->copy);
  }
  cudaMemcpyAsync(o->hCnt, &c.dCnt->npLocal, sizeof(int), cudaMemcpyDeviceToHost, o->copy);
  if (probe_dir && c.nMS > 0)
    cudaMemcpyAsync(o->hBodies, c.dBodies, sizeof(ibmdem_multisphere) * c.nMS, cudaMemcpyDeviceToHost, o->copy);
  cudaEventRecord(o->done, o->copy);
  cudaStreamWaitEvent(c.stream, o->done, 0);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("copies", e);
  const std::string tp = tecplot_path ? tecplot_path : "", pd = probe_dir ? probe_dir : "";
  const int nMS = c.nMS;
  const double rhof = c.p.rhof;
  const double centre[3] = {0.5 * (c.g.start[0] + c.g.end[0]), 0.5 * (c.g.start[1] + c.g.end[1]),
                            0.5 * (c.g.start[2] + c.g.end[2])};
  const int dev = c.device;
  o->pending = true;
  o->status = IBMDEM_OK;
  o->writer = std::thread([o, tp, pd, nMS, rhof, centre, cap, step, dev] {
    cudaSetDevice(dev);
    if (cudaEventSynchronize(o->done) != cudaSuccess) {
      o->status = IBMDEM_ECUDA;
      return;
    }
    int st = IBMDEM_OK;
    if (!tp.empty()) {
      MarkerRows m;
      m.n = *o->hCnt;
      m.stride = cap;
      m.x = o->hRows;
      m.v = o->hRows + 3 * cap;
      m.vgap = o->hRows + 6 * cap;
      m.msidx = o->hIdx;
      st = write_tecplot(tp.c_str(), m, centre);
    }
    if (!st && !pd.empty()) st = write_probes(pd.c_str(), step, nMS, o->hBodies, rhof);
    o->status = st;
  });
  return IBMDEM_OK;
}

}  // extern "C"
