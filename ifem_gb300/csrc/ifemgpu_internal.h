// Internal declarations shared by the host translation unit (host.cpp) and the
// CUDA translation units (assembly.cu, solver.cu) of libifemgpu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ifemgpu.h"

namespace ifemgpu {

constexpr int kMaxDeg = 4;        // highest polynomial degree handled
constexpr int kMaxGauss = 6;      // highest Gauss point count per direction
constexpr double kEpsZ = 1.0e-12; // singular-Jacobian tolerance (IFEM epsZ)

// Device view of one patch.  All pointers are device memory.
struct DevPatch {
  int dim;            // 2 or 3
  int p[3];           // degree per direction (0 in unused directions)
  int n[3];           // control points per direction (1 in unused)
  int nel[3];         // knot spans per direction (1 in unused)
  int ng[3];          // Gauss points per direction (1 in unused)
  int nen;            // basis functions per element
  int nq;             // Gauss points per element
  int npv;            // unknowns per node
  int kind;           // IFEMGPU_POISSON / IFEMGPU_ELASTICITY
  int rational;
  int firstNode;      // global 0-based index of the patch's first node
  const int* mlgn;    // global 0-based node of each patch node (connected models;
                      // nullptr: firstNode + node)
  double kappa, source, E, nu, body[3];
  // Lame constants and body force, formed once on the host (the FP64 pipe
  // is slow on this GPU, so no per-element divisions)
  double lam, mu;
  float lamf, muf, bodyf[3];
  double mass;        // scale of the consistent mass matrix added to K (0: none)
  int source_shape;
  const double* ctrl;     // nnod x 4: x, y, z, w (z = 0 in 2D, w = 1 if polynomial)
  const double* knots[3]; // n+p+1 per direction
  const double* logk;     // per node or nullptr
  const double* noise;    // per node or nullptr
  // 1D tables, per direction: [nel][ng][p+1] values and derivatives,
  // [nel] span lengths; filled by the basis kernel of every assembly.
  double* tabN[3];
  double* tabD[3];
  double* span[3];
  // boundary tables per direction: [side 0 = start, 1 = end][N, dN/du][p+1]
  double* tabB[3];
  // FP32 copies of tabN/tabD for the tensor-core kernel
  float* tabNf[3];
  float* tabDf[3];
  int flagBase;       // first slot of this patch's elements in the done-flag array
  int tile;           // register tile of the FP32 Poisson element matrix (2 or 4)
  // Neumann faces integrated inside the tensor-core element kernel
  int nneu;
  int neuFace[6];
  float neuT[6][3];
  int faceTables;     // face Gauss rule equals the volume rule in every direction
  // Position table of the compressed-column pattern for patches whose
  // couplings are the index box of half-width p (nullptr otherwise): for
  // node b and the box line (dz, dy), lineOff[b*(2p+1)^2 + (dz+p)(2p+1) +
  // dy+p] = (free DOFs of the box lines before it) - F(first node of the
  // line), so that row (a, k) sits in column (b, l) at
  // colptr[c] + lineOff[...] + F(a) + rank of k among a's free DOFs.
  const int* lineOff;
  // tensor-core patches: TMA tensor map (128 B) of the control net, read as
  // (p+1)^3 node boxes
  const void* tmaps;
  // tensor-core patches: element scratch (one block of elmStride floats per
  // element: element matrix and load vector, see gather.cu)
  float* elm;
  int elmStride;
  // Gauss rules: volume (gx, gw) and face (fx, fw, ngf points)
  double gx[3][kMaxGauss], gw[3][kMaxGauss];
  float gwf[3][kMaxGauss];
  double fx[3][kMaxGauss], fw[3][kMaxGauss];
  int ngf[3];
};

// Global 0-based node of patch-local node `node`.
__host__ __device__ inline int globalNode(const DevPatch& P, int node)
{
  return P.mlgn ? P.mlgn[node] : P.firstNode + node;
}

// Work item of the volume and face passes.
struct Item {
  int patch;    // index into the DevPatch array
  int elem;     // patch-local element index (first index fastest)
  int face;     // IFEM face index for Neumann items, 0 for volume items
  int bc;       // index into the Neumann value table for face items
};

struct HostBC { int face; int dofs; double value; };
// face (3D) or edge (2D) of a slave patch identified with one of a master patch
struct HostConnection { int master, mface, slave, sface, orient; };
struct HostNeumann { int face; double t[3]; };

struct HostPatch {
  int dim = 3;
  int p[3] = {0, 0, 0};
  int n[3] = {1, 1, 1};
  std::vector<double> knots[3];
  std::vector<double> ctrl4;  // nnod x 4
  bool rational = false;
  ifemgpu_material mat{};
  bool hasMat = false;
  double mass = 0.0;          // scale of the consistent mass matrix added to K
  int npv = 1;
  std::vector<double> logk, noise;
  std::vector<HostBC> bcs;
  std::vector<HostNeumann> neumann;
  // topology
  int nel[3] = {1, 1, 1};
  int nelAll = 0, nnod = 0, nelActive = 0;
  int firstNode = 0, firstElm = 0;
  std::vector<int> mlgn;     // global 0-based node of each patch node (IFEM's MLGN - 1)
  int* d_mlgn = nullptr;     // device copy for connected models
  void* d_tmaps = nullptr;   // tensor-core patches: TMA tensor map of the control net
  std::vector<char> active;  // per element: non-zero parametric volume
  int nen() const {
    return (p[0] + 1) * (p[1] + 1) * (dim == 3 ? p[2] + 1 : 1);
  }
  // device buffers owned by the patch
  double* d_ctrl = nullptr;
  double* d_stage = nullptr;  // raw coefficient upload of ifemgpu_patch_update_coefs
  double* d_knots[3] = {nullptr, nullptr, nullptr};
  double* d_logk = nullptr;
  double* d_noise = nullptr;
  double* d_tabN[3] = {nullptr, nullptr, nullptr};
  double* d_tabD[3] = {nullptr, nullptr, nullptr};
  double* d_span[3] = {nullptr, nullptr, nullptr};
  double* d_tabB[3] = {nullptr, nullptr, nullptr};
  float* d_tabNf[3] = {nullptr, nullptr, nullptr};
  float* d_tabDf[3] = {nullptr, nullptr, nullptr};
  std::vector<int> lineOff;       // see DevPatch::lineOff (empty: no box coupling)
  int* d_lineOff = nullptr;
};

constexpr int kTcElast3 = 13;  // Pass::tcDeg of the p = 3 elasticity kernel

// One colour pass of the volume or face integration.
struct Pass {
  int first;   // offset into the item array
  int count;   // items in the pass
  int face;    // 0 volume, else face pass
  int maxNd;   // largest element DOF count in the pass
  size_t smem; // dynamic shared memory of the pass' launch
  bool tc;     // volume pass on a tensor-core kernel
  int tcDeg = 0;  // 0: elasticity p = 2 kernel; 2, 3: Poisson kernel of that degree;
                  // kTcElast3: elasticity p = 3 kernel
  bool persistent = false;  // one colour-major launch ordered by done flags
  bool altColour = false;   // colour pass over a part of the persistent pass' items
};

// Test hooks of the bounded device waits (ifemgpu_debug_waits): shorter
// limits, and one element (patch index, patch-local element) whose done flag
// is never published (persistent generic pass) or whose control points are
// never copied (tensor-core kernels), so that the waits for it run out.
struct DebugWaits {
  unsigned flagSpin = 0;  // polls per neighbour-flag wait (0: default)
  unsigned mbarSpin = 0;  // polls per mbarrier wait for a copy (0: default)
  int patch = -1;
  int elem = -1;
};

// Node-wise gather launch of one (degree, npv) class of tensor-core patches:
// node item t belongs to patch pidx[r] for the last range r with start[r] <= t.
struct GatherList {
  int p = 0, npv = 0;
  bool half = false;   // each node pair summed once, written to both columns
  int* d_start = nullptr;
  int* d_pidx = nullptr;
  int nranges = 0;
  int total = 0;
  int grid = 0;
};

// tc_volume.cu
bool tcSupports(const DevPatch& P);
size_t tcVolumeSmem();

struct LearnState;  // learned.cu
struct FdState;     // fdprec.cu

}  // namespace ifemgpu

struct ifemgpu_ctx {
  ifemgpu_options opts{};
  std::string err;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<ifemgpu::HostPatch> patches;
  std::vector<ifemgpu::HostConnection> conns;  // patch connections (topology)
  bool preprocessed = false;
  bool assembled = false;
  // SAM arrays
  int nnod = 0, nel = 0, ndof = 0, neq = 0, nceq = 0;
  int64_t nnz = 0;
  std::vector<int> madof, meqn;
  std::vector<double> c0;
  std::vector<int> colptr, rowidx;
  std::vector<int> freeBefore;  // F(n): free DOFs of the nodes before node n (nnod+1)
  int* d_freeBefore = nullptr;
  // captured assembly segments: prologue, element kernels (and generic
  // volume passes), gathers, face passes
  cudaGraph_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaGraphExec_t graphExec[4] = {nullptr, nullptr, nullptr, nullptr};
  // device model
  int* d_madof = nullptr;
  int* d_meqn = nullptr;
  double* d_c0 = nullptr;
  int* d_colptr = nullptr;
  int* d_rowidx = nullptr;
  double* d_K = nullptr;
  double* d_b = nullptr;
  ifemgpu::DevPatch* d_patches = nullptr;
  std::vector<ifemgpu::DevPatch> h_devpatches;
  ifemgpu::Item* d_items = nullptr;
  double* d_neumann = nullptr;  // Neumann values, 3 per face condition
  std::vector<ifemgpu::Pass> passes;
  unsigned long long* d_counters = nullptr;  // [0] singular points
  int* d_flags = nullptr;        // per-element done flags of the persistent generic pass
  int nflags = 0;
  // tensor-core patches: element scratch and the node-wise gather launches
  float* d_elm = nullptr;
  size_t elmFloats = 0;
  std::vector<ifemgpu::GatherList> gathers;
  bool zeroSystem = true;        // some patch adds into the system (generic kernels)
  ifemgpu::DebugWaits dbg;       // test hooks of the bounded device waits
  bool checkPending = false;     // an assembly's wait counters not yet read
  // statistics of the last assembly
  double last_total_ms = 0.0, last_volume_ms = 0.0;
  unsigned long long last_singular = 0;
  int launches_per_assembly = 0;
  int assemblies = 0;  // assemblies launched (versions of K and b)
  int numSMs = 1;
  // persistent generic pass: grid (autotuned with the tile shapes at the first assembly)
  int genGrid = 0;
  bool tuned = false;
  bool useFlow = true;           // persistent pass (true) or its colour passes
  std::vector<int> tuneLog;      // (p, dim, tile) per tuned group, then (0, 0, grid)
  std::vector<char> onFlow;      // per patch: element work in the persistent pass
  // solver workspace (allocated on first solve)
  float* d_K32 = nullptr;
  short* d_off16 = nullptr;      // 16-bit column offsets of the FP32 SpMV (nullptr: 32-bit)
  int off16State = 0;            // 0 not built, 1 in use, -1 bandwidth too large
  // row-pattern dictionary of the compressed rows: rows whose column offsets
  // (col - row) form the same sequence share one int16 entry list; replaces
  // the per-entry indices in the solver's SpMVs when it is small
  int* d_rowPat = nullptr;       // neq: pattern of each row
  int* d_patStart = nullptr;     // npat + 1: start of each pattern in d_patOff
  short* d_patOff = nullptr;
  int patState = 0;              // 0 not built, 1 in use, -1 not applicable
  int numPatterns = 0;
  double* d_work = nullptr;
  size_t work_len = 0;
  double* h_pinned = nullptr;
  // captured inner-solve loops: [0] FP32 Jacobi-PCG, [1 + fine + 2 coarse] FP32
  // flexible CG (fine: 0 Jacobi, 1 Kronecker; coarse: learned correction on)
  // one captured assemble -> solve step (ifemgpu_graph_capture)
  cudaGraph_t stepGraph = nullptr;
  cudaGraphExec_t stepExec = nullptr;
  ifemgpu_solver_options stepOpts{};
  const void* stepKey = nullptr;  // workspace the step was captured on
  int stepGen = -1;
  static constexpr int kLoops = 5;
  cudaGraphExec_t loopExec[kLoops] = {};
  const void* loopKey[kLoops] = {};
  int loopGen[kLoops] = {};
  ifemgpu::FdState* fd = nullptr;  // Kronecker preconditioner (built on first use)
  int workGen = 0;               // bumped whenever the solver workspace moves
  // learned coarse correction
  ifemgpu::LearnState* learn = nullptr;
  int learnGen = 0;              // bumped by every setup
  int fieldVersion = 0;          // bumped by every field update
  double* d_rhsAlt = nullptr;    // right-hand side of a collecting solve (neq)
  // asynchronous system copies: device snapshot, copy stream, events
  int* d_basisStart = nullptr;   // per patch, first item of the basis-table launch (np + 1)
  int basisWork = 0;
  double* d_Ksnap = nullptr;
  double* d_bsnap = nullptr;
  cudaStream_t copyStream = nullptr;
  cudaEvent_t snapDone = nullptr, copyDone = nullptr;
  // solution norms and secondary solution (norms.cu): every active element
  // in patch order, its output slot in Item::bc
  ifemgpu::Item* d_normItems = nullptr;
  int nNormItems = 0, nNormSlots = 0;
  std::vector<int> normBase;     // per patch: first output slot (patch-local element e -> base + e)
  double* d_normBuf = nullptr;   // ndof solution | 2 nNormSlots element values | 2 totals
  size_t normBufLen = 0;
};

namespace ifemgpu {

ifemgpu_status setError(ifemgpu_ctx* ctx, ifemgpu_status st, const std::string& msg);
ifemgpu_status verifyAssembly(ifemgpu_ctx* ctx);
ifemgpu_status cudaFail(ifemgpu_ctx* ctx, cudaError_t e, const char* what);

// assembly.cu
ifemgpu_status uploadAssemblyModel(ifemgpu_ctx* ctx);
ifemgpu_status launchAssembly(ifemgpu_ctx* ctx);
ifemgpu_status enqueueAssembly(ifemgpu_ctx* ctx);
ifemgpu_status updateCoefs(ifemgpu_ctx* ctx, int pi, const double* coefs);

// tc_volume.cu
ifemgpu_status tcPrepare(ifemgpu_ctx* ctx);
bool tcUploadPatch(ifemgpu_ctx* ctx, HostPatch& pc, DevPatch& D);
bool nodeBoxMap(void* out, size_t esize, void* base, int inner, const int n[3], int q);
// tc_poisson.cu: tensor-core Poisson kernels (p = 2 and 3)
int tcPoissonDegree(const DevPatch& P, const HostPatch& pc);  // 2, 3 or 0 (not eligible)
bool tcPoissonUpload(ifemgpu_ctx* ctx, HostPatch& pc, DevPatch& D, int deg);
size_t tcPoissonSmem(int deg);
ifemgpu_status tcPoissonPrepare(ifemgpu_ctx* ctx);
ifemgpu_status tcPoissonLaunch(ifemgpu_ctx* ctx, const Pass& p, int deg);
ifemgpu_status tcLaunchVolume(ifemgpu_ctx* ctx, const Pass& p, int grid);
// tc_elast3.cu: tensor-core elasticity kernel, p = 3
bool tcElast3Supports(const DevPatch& P);
size_t tcElast3Smem();
ifemgpu_status tcElast3Prepare(ifemgpu_ctx* ctx);
ifemgpu_status tcElast3Launch(ifemgpu_ctx* ctx, const Pass& p);

// gather.cu
size_t elementBlockFloats(int p, int npv);
ifemgpu_status gatherPrepare(ifemgpu_ctx* ctx, GatherList& g);
ifemgpu_status gatherLaunch(ifemgpu_ctx* ctx, const GatherList& g);

// solver.cu
ifemgpu_status runSolve(ifemgpu_ctx* ctx, const ifemgpu_solver_options* o,
                        double* x, ifemgpu_solve_info* info, const double* bdev = nullptr);
ifemgpu_status captureStep(ifemgpu_ctx* ctx, const ifemgpu_solver_options* o);
ifemgpu_status launchStep(ifemgpu_ctx* ctx, double* x, ifemgpu_solve_info* info);
void dropStep(ifemgpu_ctx* ctx);
ifemgpu_status collectPairs(ifemgpu_ctx* ctx, const double* rhs, const double* xstar,
                            int stride, int maxit, double rtol, int precond);
void freeSolver(ifemgpu_ctx* ctx);
void freeNorms(ifemgpu_ctx* ctx);

// learned.cu
ifemgpu_status learnSetup(ifemgpu_ctx* ctx, int m, int nh, int capacity, unsigned seed,
                          int fieldInputs);
ifemgpu_status learnPrepare(ifemgpu_ctx* ctx);
void destroyLearn(ifemgpu_ctx* ctx);
double* learnXstar(ifemgpu_ctx* ctx);
// fine: the fine preconditioner's output for r (used by complement targets)
ifemgpu_status learnRecord(ifemgpu_ctx* ctx, const float* r, const float* x, double sx,
                           const float* fine, const float* t);
ifemgpu_status learnApply(ifemgpu_ctx* ctx, const float* r, float* z, const float* t,
                          const float* q, double* part, int nparts, unsigned* counter,
                          unsigned* counter2, double* dotOut, const double* pq, float* betaOut,
                          const double* guard);
float* learnT(ifemgpu_ctx* ctx);
ifemgpu_status learnGalerkin(ifemgpu_ctx* ctx);
ifemgpu_status learnTrain(ifemgpu_ctx* ctx, int epochs, int B, float lr, unsigned seed,
                          float* lossOut);
ifemgpu_status learnEvaluate(ifemgpu_ctx* ctx, float* mse);
ifemgpu_status learnGradients(ifemgpu_ctx* ctx, const float* X, const float* Y, int n,
                              float* gradOut, float* lossOut);
ifemgpu_status learnWeights(ifemgpu_ctx* ctx, float* theta, int* count, float* scale, int set);
int learnCount(const ifemgpu_ctx* ctx);
int learnTarget(const ifemgpu_ctx* ctx);
ifemgpu_status learnSetTarget(ifemgpu_ctx* ctx, int mode);
bool learnReady(const ifemgpu_ctx* ctx);
void learnClear(ifemgpu_ctx* ctx);

// fdprec.cu
ifemgpu_status fdSetup(ifemgpu_ctx* ctx);
void destroyFd(ifemgpu_ctx* ctx);
ifemgpu_status fdRescale(ifemgpu_ctx* ctx, const double* dinv);
// (z, q) of a flexible-CG step folded into the preconditioner's last kernel:
// partials in part (one per block), out = (z, q), beta = -(z, q) / *pq
struct FdDot {
  const float* q = nullptr;
  double* part = nullptr;
  unsigned* counter = nullptr;
  double* out = nullptr;
  const double* pq = nullptr;
  float* beta = nullptr;
};
bool fdCanDot(const ifemgpu_ctx* ctx);
ifemgpu_status fdApply(ifemgpu_ctx* ctx, const float* r, float* z, const double* guard,
                       const FdDot* dot = nullptr);
int fdLaunches(const ifemgpu_ctx* ctx);

}  // namespace ifemgpu

#define IFEMGPU_CUDA(ctx, call)                                   \
  do {                                                            \
    cudaError_t e_ = (call);                                      \
    if (e_ != cudaSuccess) return ifemgpu::cudaFail(ctx, e_, #call); \
  } while (0)

#define IFEMGPU_TRY(x)                                            \
  do {                                                            \
    ifemgpu_status s_ = (x);                                      \
    if (s_ != IFEMGPU_OK) return s_;                              \
  } while (0)
