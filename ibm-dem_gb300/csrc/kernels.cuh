// kernels.cuh — the context that owns the device-resident case state, and the
// launchers each translation unit provides.
#pragma once
#include <string>
#include <vector>

#include "common.cuh"

namespace ibmdem {

struct OutputState;  // output.cu: snapshot buffers and the file writer thread
struct FluidUpdate;  // readout.cu: the sparse field read-out

// poisson.cu: the transform grid and tables of the Poisson solve
struct PoissonPlan {
  double2* X = nullptr;   // half spectrum along x of the extended grid, x fastest
  double* aux = nullptr;  // twiddles, eigenvalues, ordered sums
  int ne[3] = {}, logn[3] = {}, nh = 0;
  size_t twOff[3] = {}, lamOff[3] = {}, partOff = 0;
  long long total = 0;
};

struct Ctx {
  ibmdem_params p{};
  Geom g{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err = "ok";
  long long launches = 0;
  size_t bytes = 0;         // device bytes this context holds
  size_t bytesParcels = 0;  // of which parcel-side buffers
  long long allocGen = 0;   // bumped whenever device buffers are replaced

  // capacities (records, images, pairs, spread contributions)
  int capLocal = 0, capImg = 0, cap = 0;
  long long capPairs = 0, capContrib = 0;

  // parcel records, double-buffered for CompressDEM
  double* recD[2] = {nullptr, nullptr};
  int* recI[2] = {nullptr, nullptr};
  int cur = 0;
  Recs rec() const { return Recs{recD[cur], recI[cur], cap}; }
  Recs recAlt() const { return Recs{recD[cur ^ 1], recI[cur ^ 1], cap}; }

  int* imgSrc = nullptr;    // [capImg] root local of each image
  int* imgShift = nullptr;  // [capImg] 2-bit shift code per axis
  int* cellStart = nullptr; // [ncell+1]
  // per-cell parcel counts of the cell-list rebuild; all zero between rebuilds
  // (the scatter zeroes the cells it used), so no sweep clears them
  int* cellCount = nullptr;  // [ncell+1]
  int* cellItems = nullptr; // [cap] part indices sorted by cell (stable)
  int* bodyStart = nullptr; // [nMS+1]
  int* bodyItems = nullptr; // [capLocal] locals grouped by body (stable)

  // scratch
  int* iTmpA = nullptr;  // [max(cap, 26*blocks)+]
  int* iTmpB = nullptr;
  int* scanScratch = nullptr;
  int* sortHist = nullptr;
  int* dTotal = nullptr;
  uint32_t* kA = nullptr;  // sort buffers [cap]
  uint32_t* vA = nullptr;
  uint32_t* kB = nullptr;
  uint32_t* vB = nullptr;

  Counters* dCnt = nullptr;
  Counters* hCnt = nullptr;  // pinned mirror

  // bodies (MS == MSGlo on one rank)
  ibmdem_multisphere* dBodies = nullptr;
  int nMS = 0, capMS = 0;
  unsigned* bodyR2 = nullptr;  // squared bounding radius (float bits)
  int* partnerCnt = nullptr;
  int* partners = nullptr;
  int maxPartners = 64;

  OutputState* out = nullptr;  // ibmdem_output_async
  FluidUpdate* upd = nullptr;  // ibmdem_update_fluid_async

  // wall probes (ibmdem_set_wall_probes): device copy with the force sums
  ibmdem_wall_probe* dProbes = nullptr;
  int nProbe = 0;

  // tangential friction of the marker contacts (ibmdem_set_friction), off while
  // ktRatio == 0.  History of the last contact-force call on side
  // Counters::histSide: per local of that call the range of its contacts, per
  // contact the partner's parcel id (I_PID; -1: not touching) and the
  // tangential displacement; pidMap takes a parcel id to that call's local.
  double ktRatio = 0.0, mu = 0.0;
  int2* histRange[2] = {};  // [capLocal]
  int* histGid[2] = {};     // [capPairs]
  double* histXi[2] = {};   // [3*capPairs]
  int* pidMap = nullptr;    // [capLocal]
  size_t bytesHist = 0;

  // contact lists
  int* activeList = nullptr;  // [capLocal]
  int* pairCnt = nullptr;     // [capLocal]
  int* pairStart = nullptr;   // [capLocal+1]
  int* pairIdx = nullptr;     // [capPairs] 0-based part indices

  // delta weights and the spread plan
  double* W = nullptr;     // [84*cap] marker-major delta weights
  int4* win = nullptr;     // [cap] cell (a,b,c) + shifted-window flags
  int4* winC = nullptr;    // [cap] the same, in cell-list order (spread plan)
  int* cntInt = nullptr;   // [cap] interior contributions per parcel
  double* fv = nullptr;    // [3*cap] fdrag*vol of locals
  uint8_t* touch = nullptr;      // touched-node flags: one bit per node, 3*nint rounded up to 128 bits
  uint32_t* planRoot = nullptr;  // [capContrib] contributing root parcel, node-major, part order
  double* planW = nullptr;       // [capContrib] its delta weight
  int* runCnt = nullptr;         // [capRuns] contributions per touched node
  unsigned long long* planAlloc = nullptr;  // (contributions << 32 | runs) reservation counter
  int* runStart = nullptr;       // [capRuns+1]
  uint32_t* runKey = nullptr;    // [capRuns]
  double* fCur = nullptr;        // [capRuns]
  double* fPrev = nullptr;       // [capRuns]
  uint32_t* lastNodes = nullptr; // [capRuns] nodes written by the last spread
  long long capRuns = 0;
  long long runsSeen = 0;  // touched nodes the host last read back (sizes the grids of the run kernels)
  bool runsSized = false;  // run arrays allocated for the counted touched nodes
  size_t bytesRuns = 0;

  // fluid
  double *u = nullptr, *v = nullptr, *w = nullptr;
  double *u0 = nullptr, *v0 = nullptr, *w0 = nullptr;
  double *fx = nullptr, *fy = nullptr, *fz = nullptr;

  // per-phase CUDA-event timing (ibmdem_timing_enable)
  bool timing = false;
  // ibmdem_step replays one captured graph per step (a one-member batch,
  // created on first use) unless stepGraphs is off or phases are being timed
  bool stepGraphs = true;
  void* stepBatch = nullptr;  // ibmdem_batch*
  struct Span {
    int phase;
    cudaEvent_t a, b;
  };
  std::vector<Span> spans;
  std::vector<cudaEvent_t> evFree;
  double phaseMs[32] = {};
  long long phaseCount[32] = {};

  // asynchronous read-out of the fields (ibmdem_get_fluid_async): later work
  // that writes them waits for the copies
  cudaEvent_t fieldsRead = nullptr;
  bool fieldsReadPending = false;
  // the MDF loop's component q finished (u|v|w and fx|fy|fz final) at
  // compDone[q]; valid while no launch followed the loop (launches == compDoneAt)
  cudaEvent_t compDone[3] = {};
  long long compDoneAt = -1;

  // fluid stencils (fluid.cu): the fields beyond u,v,w,fx,fy,fz (indexed by
  // IBMDEM_FLUID_*, allocated on first use), the guess's output (3 fields), the
  // ordered partial sums of ModifyBulkVelocity, and VelocityGuess's parameters
  double* ffield[IBMDEM_FLUID_NFIELDS] = {};
  double* fnew = nullptr;
  double* fsum = nullptr;
  double visc = 0.0, CPx = 0.0, CPy = 0.0, CPz = 0.0;

  // the Poisson solve (poisson.cu), planned on first use
  PoissonPlan pois;

  // ibmdem_set_fluid: the uploads on their own stream, beside a spread plan build
  cudaStream_t upStream = nullptr;
  cudaEvent_t upStart = nullptr, upDone[3] = {};  // upDone[q]: component q uploaded
  bool uploadPending = false;  // ibmdem_set_fluid_async: the context's stream has not waited for upDone yet

  // state flags
  bool haveFluid = false, haveParcels = false, listsBuilt = false;
  bool weightsLocal = false, weightsGhost = false, planReady = false;
  // the touched-node bits: 1 after the locals' weights cleared and marked
  // them, 2 once the images' weights added theirs (complete), 0 otherwise
  int touchState = 0;
  bool spreadValid = false;  // fCur matches the current plan
};

// timed phases (names in api.cu: ibmdem_phase_name)
enum Phase : int {
  P_INTERP = 0, P_SPREAD, P_WEIGHTS, P_PLAN, P_CELLS, P_PAIRS, P_FORCE, P_BODYSUM, P_BODYMOVE, P_MARKERS,
  P_IMAGES, P_RESET, P_FGUESS, P_FHALO, P_FOTHER, P_FPOISSON, P_COUNT
};
// records CUDA events around one phase on the context's stream (or `s`) when
// timing is on
struct PhaseScope {
  Ctx& c;
  int phase;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  PhaseScope(Ctx& ctx, int ph) : PhaseScope(ctx, ph, ctx.stream) {}
  PhaseScope(Ctx& ctx, int ph, cudaStream_t stream);
  ~PhaseScope();
};

// lists.cu
void rebuild_cell_lists(Ctx& c);
void launch_img_update(Ctx& c);
// contact.cu
void rebuild_collision_lists(Ctx& c);
// the pair forces into fcol; with friction on, also the tangential history
void launch_collision_force(Ctx& c);
// CalculateSolidBoundaryCollisionForce: wall forces into fcol (after the pair
// forces) and the probe sums; nothing without walls
void launch_wall_force(Ctx& c);
// ibm.cu
void launch_weights(Ctx& c, bool locals);
// The spread plan for the current weights, on the context's stream.
void build_spread_plan(Ctx& c);
// number of touched (component, node) pairs for the current weights; synchronises
// c.stream (-1 on a CUDA error)
long long count_touched_nodes(Ctx& c);
void launch_mdf_reset(Ctx& c, bool frozen);
// comp: one velocity component, or -1 for all three.  first: bit 0, the first
// iteration of a forcing loop whose reset is launch_mdf_stale (fdrag and fxOld
// taken as 0); bit 1, the old velocity read from the frozen field
void launch_interp(Ctx& c, int comp, int first = 0);
void launch_spread(Ctx& c, bool fused_post_guess, int comp, int first = 0);
// the forcing loop's reset when its first iteration takes the first flags:
// only the nodes the last spread wrote and the current plan does not touch
void launch_mdf_stale(Ctx& c, bool frozen);
void launch_post_guess(Ctx& c);
// The forcing loop of many frozen-fluid cases in shared launches (a batch):
// the members' descriptor table on the device and its grids.
struct ForcingBatch {
  void* desc = nullptr;
  int n = 0;
  int interpBlocksTotal = 0, spreadBlocksTotal = 0;
  int interpBlock = kBlock;
  bool anyWall = false;
};
// Bytes of the table for these members: their descriptors and the owner of
// every block of the two launches.
size_t forcing_desc_bytes(const std::vector<Ctx*>& members, int interpBlock);
// Fill the table at dDesc (forcing_desc_bytes bytes) for the members' current
// buffers and plan sizes; synchronises s (never call it while capturing).
cudaError_t forcing_desc_upload(const std::vector<Ctx*>& members, void* dDesc, int interpBlock, cudaStream_t s,
                                ForcingBatch* fb);
// One forcing iteration of every member: the interpolation for all, then the
// spread with the post-guess; first as for launch_interp (0 or 3).
void launch_forcing_batch(const ForcingBatch& fb, int first, cudaStream_t s);
void record_written_nodes(Ctx& c);
// Interpolation at n <= IBMDEM_PROBE_MAX_POINTS device points with the
// weights in a static device array (no allocation); synchronises c.stream.
// *bad = the lowest index of a point outside the box, or -1.
cudaError_t interpolate_points_noalloc(Ctx& c, int n, const double* x, double* ulp, int* bad);
// output.cu: wait for the writer thread and free the snapshot buffers
void output_release(Ctx& c);
// fluid.cu: free the fluid stencils' fields
void fluid_release(Ctx& c);
int fluid_fields(Ctx& c);     // the fluid stencils' fields, allocated on first use
void poisson_release(Ctx& c);
// readout.cu: finish a pending sparse read-out (its status), and free its buffers
int fluid_update_join(Ctx& c);
void fluid_update_release(Ctx& c);
// bodies.cu
// AssembleLocalForceMS: all twelve sums, or only the hydrodynamic (fdrag,
// fmom) or only the collision ones (fcol, fmomCol)
enum { SUMS_HYDRO = 1, SUMS_COL = 2, SUMS_ALL = 3 };
void launch_body_sums(Ctx& c, int which = SUMS_ALL);
void launch_evolution(Ctx& c);
void launch_cloud_pre(Ctx& c);
void launch_cloud_post(Ctx& c);
void launch_marker_update(Ctx& c, bool reset, bool adjust);

}  // namespace ibmdem

// the opaque handle of the C ABI
struct ibmdem_ctx {
  ibmdem::Ctx c;
};

// order the context's stream after an ibmdem_get_fluid_async still reading the fields
// and, unless only the read-out matters (uploads = false), after an
// ibmdem_set_fluid_async still uploading
inline void wait_fields_read(ibmdem::Ctx& c, bool uploads = true) {
  if (c.fieldsReadPending) {
    cudaStreamWaitEvent(c.stream, c.fieldsRead, 0);
    c.fieldsReadPending = false;
  }
  if (uploads && c.uploadPending) {
    cudaStreamWaitEvent(c.stream, c.upDone[2], 0);  // the uploads run in order on one stream
    c.uploadPending = false;
  }
}

// A frozen-fluid step (ibmdem_step) in two parts around its forcing loop, for
// a batch that runs the loop of all its members in shared launches
// (launch_forcing_batch): the plan and the reset before, the image update and
// CloudEvolutionMS after.  Both are stream-ordered on the context's stream.
int step_before_forcing(ibmdem_ctx* h);
int step_after_forcing(ibmdem_ctx* h);

// ibmdem_create with the context's allocations and work ordered on `stream`
int create_on_stream(const ibmdem_params* p, int device, cudaStream_t stream, ibmdem_ctx** out);
