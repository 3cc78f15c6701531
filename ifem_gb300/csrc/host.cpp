// host.cpp -- model input, SAM numbering and matrix pattern of libifemgpu.
//
// The numbering rules are IFEM's (see include/ifemgpu.h); the implementation
// is this library's own: node couplings of a structured patch are the index
// box of half-width p around a node, so the pattern is generated directly in
// compressed-column form, column by column in parallel, without IFEM's
// per-equation std::set (SAM::getDofCouplings, src/LinAlg/SAM.C:377-427).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <map>
#include <numeric>
#include <string>

#include "ifemgpu_internal.h"

using namespace ifemgpu;

namespace ifemgpu {

ifemgpu_status setError(ifemgpu_ctx* ctx, ifemgpu_status st, const std::string& msg)
{
  if (ctx) ctx->err = msg;
  return st;
}

ifemgpu_status cudaFail(ifemgpu_ctx* ctx, cudaError_t e, const char* what)
{
  std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  return setError(ctx, e == cudaErrorMemoryAllocation ? IFEMGPU_OUT_OF_MEMORY
                                                      : IFEMGPU_CUDA_ERROR, msg);
}

// Reads the wait counters of the last assembly once: a bounded device wait
// that gave up leaves the system invalid (IFEMGPU_DEVICE_TIMEOUT, and calls
// that need an assembled system report IFEMGPU_NOT_READY until the next
// assembly).
ifemgpu_status verifyAssembly(ifemgpu_ctx* ctx)
{
  if (!ctx->checkPending) return IFEMGPU_OK;
  ctx->checkPending = false;
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  unsigned long long c[4] = {0, 0, 0, 0};
  IFEMGPU_CUDA(ctx, cudaMemcpy(c, ctx->d_counters, sizeof(c), cudaMemcpyDeviceToHost));
  if (c[2]) {
    ctx->assembled = false;
    return setError(ctx, IFEMGPU_DEVICE_TIMEOUT,
                    "a bounded device wait gave up: the assembled system is invalid");
  }
  return IFEMGPU_OK;
}

}  // namespace ifemgpu

namespace {

void freeDevice(ifemgpu_ctx* ctx)
{
  auto f = [](void* p) { if (p) cudaFree(p); };
  for (auto& pc : ctx->patches) {
    f(pc.d_ctrl); pc.d_ctrl = nullptr;
    f(pc.d_stage); pc.d_stage = nullptr;
    f(pc.d_lineOff); pc.d_lineOff = nullptr;
    f(pc.d_logk); pc.d_logk = nullptr;
    f(pc.d_noise); pc.d_noise = nullptr;
    f(pc.d_mlgn); pc.d_mlgn = nullptr;
    f(pc.d_tmaps); pc.d_tmaps = nullptr;
    for (int d = 0; d < 3; d++) {
      f(pc.d_knots[d]); f(pc.d_tabN[d]); f(pc.d_tabD[d]); f(pc.d_span[d]); f(pc.d_tabB[d]);
      f(pc.d_tabNf[d]); f(pc.d_tabDf[d]);
      pc.d_knots[d] = pc.d_tabN[d] = pc.d_tabD[d] = pc.d_span[d] = pc.d_tabB[d] = nullptr;
      pc.d_tabNf[d] = pc.d_tabDf[d] = nullptr;
    }
  }
  f(ctx->d_madof); f(ctx->d_meqn); f(ctx->d_c0); f(ctx->d_colptr);
  f(ctx->d_rowidx); f(ctx->d_K); f(ctx->d_b); f(ctx->d_patches);
  f(ctx->d_items); f(ctx->d_neumann); f(ctx->d_counters); f(ctx->d_freeBefore);
  f(ctx->d_flags);
  f(ctx->d_basisStart);
  f(ctx->d_elm);
  for (auto& g : ctx->gathers) {
    f(g.d_start);
    f(g.d_pidx);
  }
  ctx->gathers.clear();
  ctx->d_elm = nullptr;
  ctx->elmFloats = 0;
  ctx->d_freeBefore = nullptr;
  ctx->d_flags = nullptr;
  ctx->d_basisStart = nullptr;
  for (int g = 0; g < 4; g++) {
    if (ctx->graphExec[g]) cudaGraphExecDestroy(ctx->graphExec[g]);
    if (ctx->graph[g]) cudaGraphDestroy(ctx->graph[g]);
    ctx->graphExec[g] = nullptr;
    ctx->graph[g] = nullptr;
  }
  ctx->d_madof = ctx->d_meqn = nullptr;
  ctx->d_c0 = nullptr;
  ctx->d_colptr = ctx->d_rowidx = nullptr;
  ctx->d_K = ctx->d_b = nullptr;
  ctx->d_patches = nullptr;
  ctx->d_items = nullptr;
  ctx->d_neumann = nullptr;
  ctx->d_counters = nullptr;
  dropStep(ctx);
  freeSolver(ctx);
  freeNorms(ctx);
  destroyLearn(ctx);
  destroyFd(ctx);
  f(ctx->d_rhsAlt);
  ctx->d_rhsAlt = nullptr;
}

// Patch topology: ASMs3D::generateFEMTopology (src/ASM/ASMs3D.C:487-509).
void topology(HostPatch& pc)
{
  pc.nnod = 1;
  for (int d = 0; d < 3; d++) {
    if (d >= pc.dim) { pc.p[d] = 0; pc.n[d] = 1; pc.nel[d] = 1; continue; }
    pc.nel[d] = pc.n[d] - pc.p[d];
    pc.nnod *= pc.n[d];
  }
  pc.nelAll = pc.nel[0] * pc.nel[1] * pc.nel[2];
  pc.active.assign(pc.nelAll, 0);
  pc.nelActive = 0;
  for (int e = 0; e < pc.nelAll; e++) {
    int ee[3] = {e % pc.nel[0], (e / pc.nel[0]) % pc.nel[1], e / (pc.nel[0] * pc.nel[1])};
    bool nz = true;
    for (int d = 0; d < pc.dim; d++)
      nz = nz && pc.knots[d][pc.p[d] + ee[d] + 1] > pc.knots[d][pc.p[d] + ee[d]];
    pc.active[e] = nz;
    pc.nelActive += nz;
  }
}

bool boxCoupling(const HostPatch& pc)
{
  for (char a : pc.active)
    if (!a) return false;
  return true;
}

std::vector<int> faceNodes(const HostPatch& pc, int face)
{
  std::vector<int> out;
  const int n1 = pc.n[0], n2 = pc.n[1], n3 = pc.n[2];
  const int dir = (face + 1) / 2;
  const bool hi = (face % 2) == 0;
  auto id = [&](int i, int j, int k) { return (k * n2 + j) * n1 + i; };
  if (dir == 1) {
    const int i = hi ? n1 - 1 : 0;
    for (int k = 0; k < n3; k++)
      for (int j = 0; j < n2; j++) out.push_back(id(i, j, k));
  } else if (dir == 2) {
    const int j = hi ? n2 - 1 : 0;
    for (int k = 0; k < n3; k++)
      for (int i = 0; i < n1; i++) out.push_back(id(i, j, k));
  } else {
    const int k = hi ? n3 - 1 : 0;
    for (int j = 0; j < n2; j++)
      for (int i = 0; i < n1; i++) out.push_back(id(i, j, k));
  }
  return out;
}

// DOF numbering: MADOF node-major, MSC from the boundary conditions, MEQN
// free DOFs in DOF order (SAMpatch::initNodeDofs, src/ASM/SAMpatch.C:84-161;
// SAM::initSystemEquations, src/LinAlg/SAM.C:225-336).  Fixed DOFs win over
// prescribed ones and the first prescription of a DOF wins, as IFEM's
// SAMpatch::initConstraintEqs ignores constraints on already fixed or
// constrained DOFs (src/ASM/SAMpatch.C:300-310).
// Face (3D) or edge (2D) size in IFEM's boundary-node order:
// ASMs3D::getFaceSize (src/ASM/ASMs3D.C:3796-3810).
void faceSize(const HostPatch& pc, int face, int& m1, int& m2)
{
  const int dir = (face + 1) / 2;
  if (pc.dim == 2) {
    m1 = dir == 1 ? pc.n[1] : pc.n[0];
    m2 = 1;
  } else if (dir == 1) {
    m1 = pc.n[1];
    m2 = pc.n[2];
  } else if (dir == 2) {
    m1 = pc.n[0];
    m2 = pc.n[2];
  } else {
    m1 = pc.n[0];
    m2 = pc.n[1];
  }
}

// Global node numbers (1-based, IFEM's MLGN).  Patches first get
// consecutive numbers (ASMs3D::generateFEMTopology); each connection then
// identifies the slave face's nodes with the master face's in the order and
// orientation of ASMs3D::connectBasis / ASMs2D::connectBasis
// (src/ASM/ASMs3D.C:722-796, ASMs2D.C:697-749), keeping the smaller number of
// a pair and passing the change on to the patches connected earlier
// (ASMbase::collapseNodes / mergeNodes, src/ASM/ASMbase.C:1289-1331); last,
// numbers are compacted in order of first appearance, patch by patch
// (SIMbase::renumberNodes, src/SIM/SIMbase.C:535-565, with
// ASMbase::renumberNodes and utl::renumber).  Returns the node count.
int connectAndNumber(ifemgpu_ctx* ctx, std::vector<std::vector<int>>& mlgn, std::string& err)
{
  const int np = (int)ctx->patches.size();
  std::vector<std::vector<int>> nbr(np);
  auto merge = [&](int P, int inod, int num) {
    const int old = mlgn[P][inod];
    mlgn[P][inod] = num;
    for (int Q : nbr[P])
      for (int& g : mlgn[Q])
        if (g == old) g = num;
  };
  auto collapse = [&](int M, int mnode, int S, int snode) {
    const int a = mlgn[M][mnode], b = mlgn[S][snode];
    if (a > b) merge(M, mnode, b);
    else if (b > a) merge(S, snode, a);
  };
  auto coord = [&](int P, int node, int c) {
    const HostPatch& pc = ctx->patches[P];
    const double* x = pc.ctrl4.data() + (size_t)node * 4;
    return c < pc.dim ? x[c] : 0.0;
  };
  for (const HostConnection& c : ctx->conns) {
    const int M = c.master - 1, S = c.slave - 1;
    const HostPatch &pm = ctx->patches[M], &ps = ctx->patches[S];
    const std::vector<int> mn = faceNodes(pm, c.mface), sn = faceNodes(ps, c.sface);
    int m1, m2, n1, n2;
    faceSize(ps, c.sface, m1, m2);
    faceSize(pm, c.mface, n1, n2);
    if (pm.dim == 3 && c.orient > 3) std::swap(n1, n2);
    if (n1 != m1 || n2 != m2 || mn.size() != sn.size()) {
      err = "connect: faces of different sizes";
      return -1;
    }
    if (pm.dim == 3 && c.orient > 3) std::swap(n1, n2);
    auto check = [&](int mnode, int snode) {
      for (int k = 0; k < 3; k++)
        if (std::fabs(coord(M, mnode, k) - coord(S, snode, k)) > 1.0e-4) return false;
      return true;
    };
    for (int j = 0, node = 0; j < n2; j++)
      for (int i = 0; i < n1; i++, node++) {
        int k = i, l = j;
        if (pm.dim == 3) {
          switch (c.orient) {
            case 0: k = i; l = j; break;
            case 1: k = i; l = n2 - j - 1; break;
            case 2: k = n1 - i - 1; l = j; break;
            case 3: k = n1 - i - 1; l = n2 - j - 1; break;
            case 4: k = j; l = i; break;
            case 5: k = j; l = m2 - i - 1; break;
            case 6: k = m1 - j - 1; l = i; break;
            case 7: k = m1 - j - 1; l = m2 - i - 1; break;
          }
        } else if (c.orient) {
          k = n1 - i - 1;
        }
        const int snode = sn[(size_t)l * m1 + k], mnode = mn[node];
        if (!check(mnode, snode)) {
          err = "connect: non-matching nodes (face, orientation or geometry)";
          return -1;
        }
        collapse(M, mnode, S, snode);
      }
    if (std::find(nbr[S].begin(), nbr[S].end(), M) == nbr[S].end()) {
      nbr[S].push_back(M);
      nbr[M].push_back(S);
    }
  }
  std::map<int, int> old2new;
  int runner = 0;
  for (int P = 0; P < np; P++) {
    int renum = 0;
    for (int& g : mlgn[P]) {
      auto it = old2new.find(g);
      if (it == old2new.end()) it = old2new.emplace(g, ++runner).first;
      if (g != it->second) {
        g = it->second;
        renum++;
      }
    }
    if (renum == 0 && !mlgn[P].empty())
      runner = std::max(runner, *std::max_element(mlgn[P].begin(), mlgn[P].end()));
  }
  return runner;
}

ifemgpu_status numbering(ifemgpu_ctx* ctx)
{
  int gNod = 0, gEl = 0;
  for (auto& pc : ctx->patches) {
    topology(pc);
    pc.firstNode = gNod;
    pc.firstElm = gEl;
    gNod += pc.nnod;
    gEl += pc.nelActive;
  }
  std::vector<std::vector<int>> mlgn(ctx->patches.size());
  for (size_t pi = 0; pi < ctx->patches.size(); pi++) {
    const HostPatch& pc = ctx->patches[pi];
    mlgn[pi].resize(pc.nnod);
    for (int i = 0; i < pc.nnod; i++) mlgn[pi][i] = pc.firstNode + i + 1;
  }
  if (!ctx->conns.empty()) {
    std::string err;
    gNod = connectAndNumber(ctx, mlgn, err);
    if (gNod < 0) return setError(ctx, IFEMGPU_INVALID_ARG, err);
  }
  for (size_t pi = 0; pi < ctx->patches.size(); pi++) {
    HostPatch& pc = ctx->patches[pi];
    pc.mlgn.resize(pc.nnod);
    for (int i = 0; i < pc.nnod; i++) pc.mlgn[i] = mlgn[pi][i] - 1;
  }
  ctx->nnod = gNod;
  ctx->nel = gEl;
  ctx->madof.assign(ctx->nnod + 1, 0);
  for (auto& pc : ctx->patches)
    for (int i = 0; i < pc.nnod; i++) {
      int& m = ctx->madof[pc.mlgn[i] + 1];
      if (m && m != pc.npv)
        return setError(ctx, IFEMGPU_INVALID_ARG, "connected patches with different unknowns per node");
      m = pc.npv;
    }
  ctx->madof[0] = 1;
  for (int i = 0; i < ctx->nnod; i++) ctx->madof[i + 1] += ctx->madof[i];
  ctx->ndof = ctx->madof[ctx->nnod] - 1;
  std::vector<int> msc(ctx->ndof, 1), slave(ctx->ndof, 0);
  for (auto& pc : ctx->patches)
    for (auto& bc : pc.bcs) {
      if (bc.value != 0.0) continue;
      for (int node : faceNodes(pc, bc.face))
        for (char c : std::to_string(bc.dofs)) {
          int dof = c - '0';
          if (dof >= 1 && dof <= pc.npv)
            msc[ctx->madof[pc.mlgn[node]] - 1 + dof - 1] = 0;
        }
    }
  ctx->c0.clear();
  for (auto& pc : ctx->patches)
    for (auto& bc : pc.bcs) {
      if (bc.value == 0.0) continue;
      for (int node : faceNodes(pc, bc.face))
        for (char c : std::to_string(bc.dofs)) {
          int dof = c - '0';
          if (dof < 1 || dof > pc.npv) continue;
          int idof = ctx->madof[pc.mlgn[node]] - 1 + dof - 1;
          if (msc[idof] <= 0 || slave[idof]) continue;
          ctx->c0.push_back(bc.value);
          slave[idof] = (int)ctx->c0.size();
        }
    }
  ctx->nceq = (int)ctx->c0.size();
  ctx->meqn.assign(ctx->ndof, 0);
  int ieq = 0;
  for (int i = 0; i < ctx->ndof; i++) {
    if (slave[i]) ctx->meqn[i] = -slave[i];
    else if (msc[i] == 1) ctx->meqn[i] = ++ieq;
  }
  ctx->neq = ieq;
  return IFEMGPU_OK;
}

// Coupled nodes (patch-local) of node `node`: every node sharing an element.
void coupledNodes(const HostPatch& pc, int node, std::vector<int>& out)
{
  out.clear();
  const int i = node % pc.n[0], j = (node / pc.n[0]) % pc.n[1], k = node / (pc.n[0] * pc.n[1]);
  const int lo[3] = {std::max(0, i - pc.p[0]), std::max(0, j - pc.p[1]), std::max(0, k - pc.p[2])};
  const int hi[3] = {std::min(pc.n[0] - 1, i + pc.p[0]), std::min(pc.n[1] - 1, j + pc.p[1]),
                     std::min(pc.n[2] - 1, k + pc.p[2])};
  if (boxCoupling(pc)) {
    for (int c = lo[2]; c <= hi[2]; c++)
      for (int b = lo[1]; b <= hi[1]; b++)
        for (int a = lo[0]; a <= hi[0]; a++) out.push_back((c * pc.n[1] + b) * pc.n[0] + a);
    return;
  }
  // general case: union of the node sets of the active elements around node
  const int elo[3] = {std::max(0, i - pc.p[0]), std::max(0, j - pc.p[1]), std::max(0, k - pc.p[2])};
  const int ehi[3] = {std::min(pc.nel[0] - 1, i), std::min(pc.nel[1] - 1, j), std::min(pc.nel[2] - 1, k)};
  for (int e3 = elo[2]; e3 <= ehi[2]; e3++)
    for (int e2 = elo[1]; e2 <= ehi[1]; e2++)
      for (int e1 = elo[0]; e1 <= ehi[0]; e1++) {
        int e = (e3 * pc.nel[1] + e2) * pc.nel[0] + e1;
        if (!pc.active[e]) continue;
        for (int c = 0; c <= pc.p[2]; c++)
          for (int b = 0; b <= pc.p[1]; b++)
            for (int a = 0; a <= pc.p[0]; a++)
              out.push_back(((e3 + c) * pc.n[1] + e2 + b) * pc.n[0] + e1 + a);
      }
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
}

// Compressed-column pattern, identical to SAM::getDofCouplings followed by
// SparseMatrix::optimiseCols(dofc) for patches without shared nodes.
ifemgpu_status pattern(ifemgpu_ctx* ctx)
{
  const int neq = ctx->neq;
  const bool connected = !ctx->conns.empty();
  // equation -> (patch, node, dof)
  std::vector<int> eqPatch(neq), eqNode(neq), eqGlobal(neq);
  for (int pi = 0; pi < (int)ctx->patches.size(); pi++) {
    auto& pc = ctx->patches[pi];
    for (int nd = 0; nd < pc.nnod; nd++) {
      int g = pc.mlgn[nd];
      for (int d = ctx->madof[g]; d < ctx->madof[g + 1]; d++) {
        int e = ctx->meqn[d - 1];
        if (e > 0) { eqPatch[e - 1] = pi; eqNode[e - 1] = nd; eqGlobal[e - 1] = g; }
      }
    }
  }
  // connected models: coupled global nodes of every global node, from the
  // elements of all patches (SAM::getDofCouplings, src/LinAlg/SAM.C:354-427)
  std::vector<std::vector<int>> coupled;
  if (connected) {
    coupled.resize(ctx->nnod);
    for (const auto& pc : ctx->patches) {
      const int q1 = pc.p[0] + 1, q2 = pc.p[1] + 1, q3 = pc.dim == 3 ? pc.p[2] + 1 : 1;
      std::vector<int> en;
      for (int e = 0; e < pc.nelAll; e++) {
        if (!pc.active[e]) continue;
        const int e1 = e % pc.nel[0], e2 = (e / pc.nel[0]) % pc.nel[1],
                  e3 = e / (pc.nel[0] * pc.nel[1]);
        en.clear();
        for (int c = 0; c < q3; c++)
          for (int b = 0; b < q2; b++)
            for (int a = 0; a < q1; a++)
              en.push_back(pc.mlgn[((e3 + c) * pc.n[1] + e2 + b) * pc.n[0] + e1 + a]);
        for (int g : en) coupled[g].insert(coupled[g].end(), en.begin(), en.end());
      }
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int g = 0; g < ctx->nnod; g++) {
      std::sort(coupled[g].begin(), coupled[g].end());
      coupled[g].erase(std::unique(coupled[g].begin(), coupled[g].end()), coupled[g].end());
    }
  }
  // the coupled global nodes of the node of equation c, ascending
  auto nodesOf = [&](int c, std::vector<int>& nb) {
    if (connected) {
      nb = coupled[eqGlobal[c]];
      return;
    }
    const auto& pc = ctx->patches[eqPatch[c]];
    coupledNodes(pc, eqNode[c], nb);
    for (int& m : nb) m = pc.mlgn[m];
  };
  // column counts (columns of one node share their row set)
  std::vector<int64_t> cnt(neq + 1, 0);
#pragma omp parallel
  {
    std::vector<int> nb;
#pragma omp for schedule(dynamic, 256)
    for (int c = 0; c < neq; c++) {
      nodesOf(c, nb);
      int64_t s = 0;
      for (int g : nb)
        for (int d = ctx->madof[g]; d < ctx->madof[g + 1]; d++) s += ctx->meqn[d - 1] > 0;
      cnt[c + 1] = s;
    }
  }
  for (int c = 0; c < neq; c++) cnt[c + 1] += cnt[c];
  if (cnt[neq] >= (int64_t)INT32_MAX)
    return setError(ctx, IFEMGPU_UNSUPPORTED, "matrix has more than 2^31-1 non-zeros");
  ctx->nnz = cnt[neq];
  ctx->colptr.resize(neq + 1);
  for (int c = 0; c <= neq; c++) ctx->colptr[c] = (int)cnt[c];
  ctx->rowidx.resize(ctx->nnz);
#pragma omp parallel
  {
    std::vector<int> nb;
#pragma omp for schedule(dynamic, 256)
    for (int c = 0; c < neq; c++) {
      nodesOf(c, nb);
      int64_t k = cnt[c];
      for (int g : nb)
        for (int d = ctx->madof[g]; d < ctx->madof[g + 1]; d++)
          if (ctx->meqn[d - 1] > 0) ctx->rowidx[k++] = ctx->meqn[d - 1] - 1;
    }
  }
  // F(n), and the line-offset tables that give pattern positions without a
  // search for patches whose couplings are the index box
  ctx->freeBefore.assign(ctx->nnod + 1, 0);
  for (int n = 0; n < ctx->nnod; n++) {
    int f = 0;
    for (int d = ctx->madof[n]; d < ctx->madof[n + 1]; d++) f += ctx->meqn[d - 1] > 0;
    ctx->freeBefore[n + 1] = ctx->freeBefore[n] + f;
  }
  const std::vector<int>& F = ctx->freeBefore;
  for (auto& pc : ctx->patches) {
    pc.lineOff.clear();
    if (!boxCoupling(pc) || connected) continue;  // connected: positions by search
    const int w1 = 2 * pc.p[1] + 1, w2 = 2 * pc.p[2] + 1;
    pc.lineOff.assign((size_t)pc.nnod * w1 * w2, 0);
#pragma omp parallel for schedule(static)
    for (int b = 0; b < pc.nnod; b++) {
      const int xb = b % pc.n[0], yb = (b / pc.n[0]) % pc.n[1], zb = b / (pc.n[0] * pc.n[1]);
      const int x0 = std::max(0, xb - pc.p[0]), x1 = std::min(pc.n[0] - 1, xb + pc.p[0]);
      int acc = 0;
      for (int dz = -pc.p[2]; dz <= pc.p[2]; dz++) {
        const int z = zb + dz;
        if (z < 0 || z >= pc.n[2]) continue;
        for (int dy = -pc.p[1]; dy <= pc.p[1]; dy++) {
          const int y = yb + dy;
          if (y < 0 || y >= pc.n[1]) continue;
          const int s = pc.firstNode + (z * pc.n[1] + y) * pc.n[0] + x0;
          const int e = pc.firstNode + (z * pc.n[1] + y) * pc.n[0] + x1 + 1;
          pc.lineOff[(size_t)b * w1 * w2 + (dz + pc.p[2]) * w1 + dy + pc.p[1]] = acc - F[s];
          acc += F[e] - F[s];
        }
      }
    }
  }
  return IFEMGPU_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

int ifemgpu_abi_version(void) { return IFEMGPU_ABI_VERSION; }

ifemgpu_status ifemgpu_ctx_create(ifemgpu_ctx** out, const ifemgpu_options* opts)
{
  if (!out) return IFEMGPU_INVALID_ARG;
  *out = nullptr;
  ifemgpu_ctx* ctx = new ifemgpu_ctx;
  if (opts) ctx->opts = *opts;
  else { ctx->opts.device = 0; ctx->opts.ke_precision = IFEMGPU_KE_FP64; ctx->opts.n_gauss = 4; }
  if (ctx->opts.device < 0) {  // host-only: numbering and pattern, no device work
    *out = ctx;
    return IFEMGPU_OK;
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    delete ctx;
    return IFEMGPU_CUDA_ERROR;
  }
  if (ctx->opts.device < 0 || ctx->opts.device >= ndev) { delete ctx; return IFEMGPU_INVALID_ARG; }
  if (cudaSetDevice(ctx->opts.device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return IFEMGPU_CUDA_ERROR;
  }
  for (auto& ev : ctx->ev) cudaEventCreate(&ev);
  *out = ctx;
  return IFEMGPU_OK;
}

void ifemgpu_ctx_destroy(ifemgpu_ctx* ctx)
{
  if (!ctx) return;
  if (ctx->opts.device >= 0) {
    cudaSetDevice(ctx->opts.device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    freeDevice(ctx);
    for (auto& ev : ctx->ev) if (ev) cudaEventDestroy(ev);
    if (ctx->copyStream) {
      cudaStreamSynchronize(ctx->copyStream);
      cudaStreamDestroy(ctx->copyStream);
    }
    if (ctx->snapDone) cudaEventDestroy(ctx->snapDone);
    if (ctx->copyDone) cudaEventDestroy(ctx->copyDone);
    if (ctx->d_Ksnap) cudaFree(ctx->d_Ksnap);
    if (ctx->d_bsnap) cudaFree(ctx->d_bsnap);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
  }
  delete ctx;
}

const char* ifemgpu_last_error(const ifemgpu_ctx* ctx)
{
  return ctx ? ctx->err.c_str() : "null context";
}

ifemgpu_status ifemgpu_patch_add(ifemgpu_ctx* ctx, int dim, const int* degree,
                                 const int* ncoef, const double* const* knots,
                                 const double* coefs, int rational, int* patch_id)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (ctx->preprocessed) return setError(ctx, IFEMGPU_INVALID_ARG, "model already preprocessed");
  if ((dim != 2 && dim != 3) || !degree || !ncoef || !knots || !coefs)
    return setError(ctx, IFEMGPU_INVALID_ARG, "patch_add: bad dimension or null array");
  HostPatch pc;
  pc.dim = dim;
  int nn = 1;
  for (int d = 0; d < dim; d++) {
    if (degree[d] < 1 || degree[d] > kMaxDeg)
      return setError(ctx, IFEMGPU_UNSUPPORTED, "patch_add: degree must be in 1..4");
    if (ncoef[d] < degree[d] + 1 || !knots[d])
      return setError(ctx, IFEMGPU_INVALID_ARG, "patch_add: too few control points");
    pc.p[d] = degree[d];
    pc.n[d] = ncoef[d];
    pc.knots[d].assign(knots[d], knots[d] + ncoef[d] + degree[d] + 1);
    for (size_t i = 1; i < pc.knots[d].size(); i++)
      if (pc.knots[d][i] < pc.knots[d][i - 1])
        return setError(ctx, IFEMGPU_INVALID_ARG, "patch_add: decreasing knot vector");
    nn *= ncoef[d];
  }
  const int stride = dim + (rational ? 1 : 0);
  pc.rational = rational != 0;
  pc.ctrl4.assign((size_t)nn * 4, 0.0);
  for (int i = 0; i < nn; i++) {
    for (int c = 0; c < dim; c++) pc.ctrl4[(size_t)i * 4 + c] = coefs[(size_t)i * stride + c];
    pc.ctrl4[(size_t)i * 4 + 3] = rational ? coefs[(size_t)i * stride + dim] : 1.0;
    if (!(pc.ctrl4[(size_t)i * 4 + 3] > 0.0))
      return setError(ctx, IFEMGPU_INVALID_ARG, "patch_add: weights must be positive");
  }
  pc.nnod = nn;
  ctx->patches.push_back(std::move(pc));
  if (patch_id) *patch_id = (int)ctx->patches.size();
  return IFEMGPU_OK;
}

static HostPatch* getPatch(ifemgpu_ctx* ctx, int pid)
{
  if (!ctx || pid < 1 || pid > (int)ctx->patches.size()) return nullptr;
  return &ctx->patches[pid - 1];
}

ifemgpu_status ifemgpu_patch_set_material(ifemgpu_ctx* ctx, int patch_id,
                                          const ifemgpu_material* mat)
{
  HostPatch* pc = getPatch(ctx, patch_id);
  if (!pc || !mat) return setError(ctx, IFEMGPU_INVALID_ARG, "set_material: bad patch or material");
  if (ctx->preprocessed) return setError(ctx, IFEMGPU_INVALID_ARG, "model already preprocessed");
  if (mat->kind == IFEMGPU_ELASTICITY && pc->dim != 3)
    return setError(ctx, IFEMGPU_UNSUPPORTED, "elasticity is implemented for 3D patches");
  if (mat->kind != IFEMGPU_POISSON && mat->kind != IFEMGPU_ELASTICITY)
    return setError(ctx, IFEMGPU_INVALID_ARG, "set_material: unknown kind");
  pc->mat = *mat;
  pc->hasMat = true;
  pc->npv = mat->kind == IFEMGPU_ELASTICITY ? pc->dim : 1;
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_patch_connect(ifemgpu_ctx* ctx, int master, int master_face, int slave,
                                     int slave_face, int orient)
{
  HostPatch* pm = getPatch(ctx, master);
  HostPatch* ps = getPatch(ctx, slave);
  if (!pm || !ps || master == slave || pm->dim != ps->dim)
    return setError(ctx, IFEMGPU_INVALID_ARG, "connect: bad patches");
  const int nf = 2 * pm->dim;
  if (master_face < 1 || master_face > nf || slave_face < 1 || slave_face > nf || orient < 0 ||
      orient > (pm->dim == 3 ? 7 : 1))
    return setError(ctx, IFEMGPU_INVALID_ARG, "connect: bad face or orientation");
  if (ctx->preprocessed) return setError(ctx, IFEMGPU_INVALID_ARG, "model already preprocessed");
  ctx->conns.push_back({master, master_face, slave, slave_face, orient});
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_patch_set_mass(ifemgpu_ctx* ctx, int patch_id, double scale)
{
  HostPatch* pc = getPatch(ctx, patch_id);
  if (!pc || !std::isfinite(scale)) return setError(ctx, IFEMGPU_INVALID_ARG, "set_mass: bad patch or scale");
  if (ctx->preprocessed) return setError(ctx, IFEMGPU_INVALID_ARG, "model already preprocessed");
  pc->mass = scale;
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_patch_set_field(ifemgpu_ctx* ctx, int patch_id, int which,
                                       const double* values)
{
  HostPatch* pc = getPatch(ctx, patch_id);
  if (!pc || !values) return setError(ctx, IFEMGPU_INVALID_ARG, "set_field: bad patch or values");
  if (ctx->preprocessed) return setError(ctx, IFEMGPU_INVALID_ARG, "model already preprocessed");
  int nn = (int)(pc->ctrl4.size() / 4);
  if (which == IFEMGPU_FIELD_LOG_KAPPA) pc->logk.assign(values, values + nn);
  else if (which == IFEMGPU_FIELD_SOURCE_NOISE) pc->noise.assign(values, values + nn);
  else return setError(ctx, IFEMGPU_INVALID_ARG, "set_field: unknown field");
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_patch_constrain_face(ifemgpu_ctx* ctx, int patch_id, int face,
                                            int dofs, double value)
{
  HostPatch* pc = getPatch(ctx, patch_id);
  if (!pc || face < 1 || face > 2 * pc->dim || dofs < 1)
    return setError(ctx, IFEMGPU_INVALID_ARG, "constrain_face: bad patch, face or dofs");
  if (ctx->preprocessed) return setError(ctx, IFEMGPU_INVALID_ARG, "model already preprocessed");
  pc->bcs.push_back({face, dofs, value});
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_patch_add_neumann(ifemgpu_ctx* ctx, int patch_id, int face,
                                         const double* values)
{
  HostPatch* pc = getPatch(ctx, patch_id);
  if (!pc || face < 1 || face > 2 * pc->dim || !values)
    return setError(ctx, IFEMGPU_INVALID_ARG, "add_neumann: bad patch, face or values");
  if (pc->dim != 3) return setError(ctx, IFEMGPU_UNSUPPORTED, "Neumann faces need 3D patches");
  if (!pc->hasMat) return setError(ctx, IFEMGPU_NOT_READY, "add_neumann: set the material first");
  if (ctx->preprocessed) return setError(ctx, IFEMGPU_INVALID_ARG, "model already preprocessed");
  HostNeumann nm{face, {0, 0, 0}};
  for (int c = 0; c < pc->npv; c++) nm.t[c] = values[c];
  pc->neumann.push_back(nm);
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_preprocess(ifemgpu_ctx* ctx)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (ctx->preprocessed) return setError(ctx, IFEMGPU_INVALID_ARG, "already preprocessed");
  if (ctx->patches.empty()) return setError(ctx, IFEMGPU_NOT_READY, "no patches");
  for (auto& pc : ctx->patches)
    if (!pc.hasMat) return setError(ctx, IFEMGPU_NOT_READY, "patch without material");
  ifemgpu_status st = numbering(ctx);
  if (st != IFEMGPU_OK) return st;
  st = pattern(ctx);
  if (st != IFEMGPU_OK) return st;
  if (ctx->opts.device >= 0) {
    IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
    st = uploadAssemblyModel(ctx);
    if (st != IFEMGPU_OK) { freeDevice(ctx); return st; }
  }
  ctx->preprocessed = true;
  if (ctx->opts.verbose)
    std::printf("\n >>> SAM model summary <<<\nNumber of elements    %d\nNumber of nodes       %d\n"
                "Number of dofs        %d\nNumber of unknowns    %d\nNon-zeroes            %lld\n",
                ctx->nel, ctx->nnod, ctx->ndof, ctx->neq, (long long)ctx->nnz);
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_get_sizes(const ifemgpu_ctx* ctx, ifemgpu_sizes* out)
{
  if (!ctx || !out) return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed) return IFEMGPU_NOT_READY;
  out->npatch = (int)ctx->patches.size();
  out->nnod = ctx->nnod;
  out->nel = ctx->nel;
  out->ndof = ctx->ndof;
  out->neq = ctx->neq;
  out->nceq = ctx->nceq;
  out->nnz = ctx->nnz;
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_get_madof(const ifemgpu_ctx* ctx, int* madof)
{
  if (!ctx || !madof) return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed) return IFEMGPU_NOT_READY;
  std::memcpy(madof, ctx->madof.data(), sizeof(int) * ctx->madof.size());
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_get_meqn(const ifemgpu_ctx* ctx, int* meqn)
{
  if (!ctx || !meqn) return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed) return IFEMGPU_NOT_READY;
  std::memcpy(meqn, ctx->meqn.data(), sizeof(int) * ctx->meqn.size());
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_get_mnpc(const ifemgpu_ctx* ctx, int patch_id, int* mnpc)
{
  if (!ctx || !mnpc || patch_id < 1 || patch_id > (int)ctx->patches.size())
    return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed) return IFEMGPU_NOT_READY;
  const HostPatch& pc = ctx->patches[patch_id - 1];
  const int q1 = pc.p[0] + 1, q2 = pc.p[1] + 1, q3 = pc.p[2] + 1;
  size_t k = 0;
  for (int e = 0; e < pc.nelAll; e++) {
    const int e1 = e % pc.nel[0], e2 = (e / pc.nel[0]) % pc.nel[1], e3 = e / (pc.nel[0] * pc.nel[1]);
    for (int c = 0; c < q3; c++)
      for (int b = 0; b < q2; b++)
        for (int a = 0; a < q1; a++)
          mnpc[k++] = pc.active[e] ? ((e3 + c) * pc.n[1] + e2 + b) * pc.n[0] + e1 + a : -1;
  }
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_get_pattern(const ifemgpu_ctx* ctx, int* colptr, int* rowidx)
{
  if (!ctx || !colptr || !rowidx) return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed) return IFEMGPU_NOT_READY;
  std::memcpy(colptr, ctx->colptr.data(), sizeof(int) * ctx->colptr.size());
  std::memcpy(rowidx, ctx->rowidx.data(), sizeof(int) * ctx->rowidx.size());
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_patch_update_coefs(ifemgpu_ctx* ctx, int patch_id, const double* coefs)
{
  HostPatch* pc = getPatch(ctx, patch_id);
  if (!pc || !coefs) return setError(ctx, IFEMGPU_INVALID_ARG, "update_coefs: bad patch or array");
  if (!ctx->preprocessed || ctx->opts.device < 0)
    return setError(ctx, IFEMGPU_NOT_READY, "update_coefs before preprocess");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  return updateCoefs(ctx, patch_id - 1, coefs);
}

ifemgpu_status ifemgpu_get_stream(const ifemgpu_ctx* ctx, void** stream)
{
  if (!ctx || !stream) return IFEMGPU_INVALID_ARG;
  *stream = (void*)ctx->stream;
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_assemble(ifemgpu_ctx* ctx, int sync)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed) return setError(ctx, IFEMGPU_NOT_READY, "assemble before preprocess");
  if (ctx->opts.device < 0) return setError(ctx, IFEMGPU_NOT_READY, "host-only context (device -1)");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  ifemgpu_status st = launchAssembly(ctx);
  if (st != IFEMGPU_OK) return st;
  ctx->assembled = true;
  ctx->checkPending = true;
  return sync ? verifyAssembly(ctx) : IFEMGPU_OK;
}

ifemgpu_status ifemgpu_debug_waits(ifemgpu_ctx* ctx, unsigned flag_spin, unsigned copy_spin,
                                   int patch_id, int element)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (patch_id < 0 || patch_id > (int)ctx->patches.size() || (patch_id > 0 && element < 0))
    return setError(ctx, IFEMGPU_INVALID_ARG, "debug_waits: bad patch or element");
  ctx->dbg.flagSpin = flag_spin;
  ctx->dbg.mbarSpin = copy_spin;
  ctx->dbg.patch = patch_id - 1;
  ctx->dbg.elem = patch_id > 0 ? element : -1;
  // the captured kernel sequences hold the old parameters
  for (int g = 0; g < 4; g++) {
    if (ctx->graphExec[g]) cudaGraphExecDestroy(ctx->graphExec[g]);
    if (ctx->graph[g]) cudaGraphDestroy(ctx->graph[g]);
    ctx->graphExec[g] = nullptr;
    ctx->graph[g] = nullptr;
  }
  dropStep(ctx);
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_last_assembly_phases(ifemgpu_ctx* ctx, double* element_ms,
                                            double* gather_ms)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "no assembly yet");
  IFEMGPU_TRY(verifyAssembly(ctx));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  float t0 = 0.f, t1 = 0.f;
  IFEMGPU_CUDA(ctx, cudaEventElapsedTime(&t0, ctx->ev[1], ctx->ev[2]));
  IFEMGPU_CUDA(ctx, cudaEventElapsedTime(&t1, ctx->ev[2], ctx->ev[3]));
  if (element_ms) *element_ms = t0;
  if (gather_ms) *gather_ms = t1;
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_last_assembly_stats(ifemgpu_ctx* ctx, double* total_ms,
                                           double* volume_ms, long long* singular,
                                           int* kernel_launches)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "no assembly yet");
  IFEMGPU_TRY(verifyAssembly(ctx));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  float t0 = 0.f, t1 = 0.f;
  IFEMGPU_CUDA(ctx, cudaEventElapsedTime(&t0, ctx->ev[0], ctx->ev[4]));
  IFEMGPU_CUDA(ctx, cudaEventElapsedTime(&t1, ctx->ev[1], ctx->ev[3]));
  unsigned long long s = 0;
  IFEMGPU_CUDA(ctx, cudaMemcpy(&s, ctx->d_counters, sizeof(s), cudaMemcpyDeviceToHost));
  if (total_ms) *total_ms = t0;
  if (volume_ms) *volume_ms = t1;
  if (singular) *singular = (long long)s;
  if (kernel_launches) *kernel_launches = ctx->launches_per_assembly;
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_copy_matrix(ifemgpu_ctx* ctx, double* values)
{
  if (!ctx || !values) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "no assembly yet");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  IFEMGPU_TRY(verifyAssembly(ctx));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(values, ctx->d_K, sizeof(double) * ctx->nnz,
                                    cudaMemcpyDeviceToHost, ctx->stream));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_copy_system_async(ifemgpu_ctx* ctx, double* values, double* rhs)
{
  if (!ctx || !values) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "no assembly yet");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  if (!ctx->copyStream) {
    IFEMGPU_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copyStream, cudaStreamNonBlocking));
    IFEMGPU_CUDA(ctx, cudaEventCreateWithFlags(&ctx->snapDone, cudaEventDisableTiming));
    IFEMGPU_CUDA(ctx, cudaEventCreateWithFlags(&ctx->copyDone, cudaEventDisableTiming));
    IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_Ksnap, sizeof(double) * std::max<int64_t>(ctx->nnz, 1)));
    IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_bsnap, sizeof(double) * std::max(ctx->neq, 1)));
    IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->copyDone, ctx->copyStream));
  }
  // the snapshot is overwritten only after the previous copy has drained it
  IFEMGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->copyDone, 0));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(ctx->d_Ksnap, ctx->d_K, sizeof(double) * ctx->nnz,
                                    cudaMemcpyDeviceToDevice, ctx->stream));
  if (rhs)
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(ctx->d_bsnap, ctx->d_b, sizeof(double) * ctx->neq,
                                      cudaMemcpyDeviceToDevice, ctx->stream));
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->snapDone, ctx->stream));
  IFEMGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->copyStream, ctx->snapDone, 0));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(values, ctx->d_Ksnap, sizeof(double) * ctx->nnz,
                                    cudaMemcpyDeviceToHost, ctx->copyStream));
  if (rhs)
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(rhs, ctx->d_bsnap, sizeof(double) * ctx->neq,
                                      cudaMemcpyDeviceToHost, ctx->copyStream));
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->copyDone, ctx->copyStream));
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_copy_wait(ifemgpu_ctx* ctx)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (ctx->copyStream) IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->copyStream));
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_copy_rhs(ifemgpu_ctx* ctx, double* rhs)
{
  if (!ctx || !rhs) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "no assembly yet");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  IFEMGPU_TRY(verifyAssembly(ctx));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(rhs, ctx->d_b, sizeof(double) * ctx->neq,
                                    cudaMemcpyDeviceToHost, ctx->stream));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return IFEMGPU_OK;
}

namespace {

// Writer of the text formats of IFEM's SparseMatrix::dump (SuperLU layout)
// and StdVector::dump; the character sequence follows those functions so
// that dumps compare byte for byte.
bool writeMatrix(std::ostream& os, int n, const int* IA, const int* JA, const double* A, int format)
{
  const int nnz = IA[n];
  std::string end;
  if (format == IFEMGPU_DUMP_MATRIX_MARKET) {
    os << "%%MatrixMarket matrix coordinate real general\n% label = A\n";
    os << n << ' ' << n << ' ' << nnz << '\n';
    end = "\n";
  } else if (format == IFEMGPU_DUMP_MATLAB) {
    os << "A = [\n";
    end = ";\n";
  } else if (format == IFEMGPU_DUMP_FLAT) {  // SparseMatrix::write
    os << "A = [\n";
    os << n << ' ' << n << ' ' << nnz << '\n';
    for (int i = 0; i < nnz; i++) os << A[i] << ' ';
    os << '\n' << n + 1 << '\n';
    for (int i = 0; i <= n; i++) os << IA[i] << ' ';
    os << '\n' << nnz << '\n';
    for (int i = 0; i < nnz; i++) os << JA[i] << ' ';
    os << std::endl << "]\n";
    return bool(os);
  } else {
    return false;
  }
  if (nnz > 0) {
    os << JA[0] + 1 << " 1 " << A[0];
    for (int j = 1; j <= n; j++)
      for (int i = IA[j - 1]; i < IA[j]; i++)
        if (j > 1 || i != IA[0]) os << end << JA[i] + 1 << ' ' << j << ' ' << A[i];
  }
  if (format == IFEMGPU_DUMP_MATLAB) os << "]";
  os << end;
  return bool(os);
}

bool writeVector(std::ostream& os, int n, const double* x, int format, double tol)
{
  auto trunc = [tol](double v) { return v > tol || v < -tol || std::isnan(v) ? v : 0.0; };
  if (format == IFEMGPU_DUMP_MATLAB) {  // utl::writeMatlab
    os << "b = [";
    for (int i = 0; i < n; i++) os << ' ' << trunc(x[i]);
    os << " ];" << std::endl;
  } else if (format == IFEMGPU_DUMP_MATRIX_MARKET) {
    os << "%%MatrixMarket matrix array real general\n" << n << " 1";
    for (int i = 0; i < n; i++) os << '\n' << x[i];
    os << std::endl;
  } else if (format == IFEMGPU_DUMP_FLAT) {  // operator<< of utl::vector, 6 per line
    os << "b =";
    if (n < 1) os << " (empty)";
    for (int i = 0; i < n; i++) os << ((i % 6) ? ' ' : '\n') << trunc(x[i]);
    os << std::endl;
  } else {
    return false;
  }
  return bool(os);
}

}  // namespace

ifemgpu_status ifemgpu_write_system(int n, const int* colptr, const int* rowidx,
                                    const double* values, const double* rhs,
                                    const char* matrix_path, const char* rhs_path,
                                    int format, double zero_tol)
{
  if (n < 0 || (matrix_path && (!colptr || !rowidx || !values)) || (rhs_path && !rhs) ||
      format < IFEMGPU_DUMP_FLAT || format > IFEMGPU_DUMP_MATRIX_MARKET)
    return IFEMGPU_INVALID_ARG;
  if (matrix_path) {
    std::ofstream os(matrix_path);
    os << std::setprecision(17);
    if (!os || !writeMatrix(os, n, colptr, rowidx, values, format)) return IFEMGPU_INVALID_ARG;
  }
  if (rhs_path) {
    std::ofstream os(rhs_path);
    os << std::setprecision(17);
    if (!os || !writeVector(os, n, rhs, format, zero_tol)) return IFEMGPU_INVALID_ARG;
  }
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_dump_system(ifemgpu_ctx* ctx, const char* matrix_path,
                                   const char* rhs_path, int format, double zero_tol)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "no assembly yet");
  std::vector<double> A(matrix_path ? ctx->nnz : 0), b(rhs_path ? ctx->neq : 0);
  ifemgpu_status st = IFEMGPU_OK;
  if (matrix_path && (st = ifemgpu_copy_matrix(ctx, A.data())) != IFEMGPU_OK) return st;
  if (rhs_path && (st = ifemgpu_copy_rhs(ctx, b.data())) != IFEMGPU_OK) return st;
  st = ifemgpu_write_system(ctx->neq, ctx->colptr.data(), ctx->rowidx.data(), A.data(), b.data(),
                            matrix_path, rhs_path, format, zero_tol);
  if (st != IFEMGPU_OK) return setError(ctx, st, "dump_system: bad format or unwritable path");
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_device_system(ifemgpu_ctx* ctx, const double** values,
                                     const int** colptr, const int** rowidx,
                                     const double** rhs)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed) return setError(ctx, IFEMGPU_NOT_READY, "not preprocessed");
  if (values) *values = ctx->d_K;
  if (colptr) *colptr = ctx->d_colptr;
  if (rowidx) *rowidx = ctx->d_rowidx;
  if (rhs) *rhs = ctx->d_b;
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_solve(ifemgpu_ctx* ctx, const ifemgpu_solver_options* opts,
                             double* x, ifemgpu_solve_info* info)
{
  if (!ctx || !opts || !x) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "solve before assemble");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  IFEMGPU_TRY(verifyAssembly(ctx));
  return runSolve(ctx, opts, x, info);
}

ifemgpu_status ifemgpu_expand_solution(const ifemgpu_ctx* ctx, const double* x,
                                       double* u, double scale)
{
  if (!ctx || !x || !u) return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed) return IFEMGPU_NOT_READY;
  for (int i = 0; i < ctx->ndof; i++) {
    int e = ctx->meqn[i];
    u[i] = e > 0 ? x[e - 1] : (e < 0 ? ctx->c0[-e - 1] * scale : 0.0);
  }
  return IFEMGPU_OK;
}

// Block-CSR copy of the assembled matrix: block rows of `block` consecutive
// equations that are the DOFs of one node.  The pattern is symmetric, so the
// block columns of block row I are the block rows listed in column I b; the
// value of block (I, J)[k][l] = K(I b + k, J b + l) is read from column
// J b + l at row I b + k (the values themselves are symmetric only up to
// rounding).
ifemgpu_status ifemgpu_copy_matrix_bsr(ifemgpu_ctx* ctx, int block, int* nbrows, int64_t* nnzb,
                                       int* browptr, int* bcolind, double* bvals)
{
  if (!ctx || block < 1) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "copy_matrix_bsr before assemble");
  const int b = block, neq = ctx->neq;
  if (neq % b) return setError(ctx, IFEMGPU_UNSUPPORTED, "copy_matrix_bsr: equations not a multiple of the block");
  // equation -> (node, component); blocks must be the DOFs 0..b-1 of one node
  std::vector<int> eqNode(neq, -1), eqComp(neq, -1);
  for (int n = 0; n < ctx->nnod; n++)
    for (int d = ctx->madof[n] - 1; d < ctx->madof[n + 1] - 1; d++) {
      const int e = ctx->meqn[d];
      if (e > 0) { eqNode[e - 1] = n; eqComp[e - 1] = d - (ctx->madof[n] - 1); }
    }
  const int nb = neq / b;
  for (int I = 0; I < nb; I++)
    for (int k = 0; k < b; k++) {
      const int e = I * b + k;
      if (eqComp[e] != k || eqNode[e] != eqNode[I * b])
        return setError(ctx, IFEMGPU_UNSUPPORTED, "copy_matrix_bsr: a node's DOFs are not one free block");
      const int c0 = ctx->colptr[I * b], c = ctx->colptr[e];
      const int len = ctx->colptr[I * b + 1] - c0;
      if (ctx->colptr[e + 1] - c != len ||
          !std::equal(ctx->rowidx.begin() + c0, ctx->rowidx.begin() + c0 + len, ctx->rowidx.begin() + c))
        return setError(ctx, IFEMGPU_UNSUPPORTED, "copy_matrix_bsr: DOFs of a node couple differently");
      if (len % b) return setError(ctx, IFEMGPU_UNSUPPORTED, "copy_matrix_bsr: partial blocks");
    }
  if (nbrows) *nbrows = nb;
  if (nnzb) *nnzb = ctx->nnz / ((int64_t)b * b);
  if (!browptr && !bcolind && !bvals) return IFEMGPU_OK;
  std::vector<double> K;
  if (bvals) {
    K.resize(ctx->nnz);
    ifemgpu_status st = ifemgpu_copy_matrix(ctx, K.data());
    if (st != IFEMGPU_OK) return st;
  }
  int64_t blk = 0;
  if (browptr) browptr[0] = 0;
  for (int I = 0; I < nb; I++) {
    const int c0 = ctx->colptr[I * b], len = ctx->colptr[I * b + 1] - c0;
    for (int p = 0; p < len; p += b, blk++) {
      const int J = ctx->rowidx[c0 + p] / b;
      if (bcolind) bcolind[blk] = J;
      if (!bvals) continue;
      // position of row I b in column J b (same offset in columns J b + l)
      const int* col = ctx->rowidx.data() + ctx->colptr[J * b];
      const int clen = ctx->colptr[J * b + 1] - ctx->colptr[J * b];
      const int q = (int)(std::lower_bound(col, col + clen, I * b) - col);
      for (int k = 0; k < b; k++)
        for (int l = 0; l < b; l++)
          bvals[blk * b * b + k * b + l] = K[ctx->colptr[J * b + l] + q + k];
    }
    if (browptr) browptr[I + 1] = (int)blk;
  }
  return IFEMGPU_OK;
}

// ---- learned coarse correction (learned.cu, solver.cu) ----------------------

static ifemgpu_status deviceReady(ifemgpu_ctx* ctx)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed) return setError(ctx, IFEMGPU_NOT_READY, "not preprocessed");
  if (ctx->opts.device < 0) return setError(ctx, IFEMGPU_NOT_READY, "host-only context (device -1)");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_learn_setup(ifemgpu_ctx* ctx, const ifemgpu_learn_options* o)
{
  ifemgpu_status st = deviceReady(ctx);
  if (st != IFEMGPU_OK) return st;
  if (!o) return setError(ctx, IFEMGPU_INVALID_ARG, "learn_setup: null options");
  return learnSetup(ctx, o->coarse_cells, o->hidden, o->capacity, o->seed, o->field_inputs);
}

ifemgpu_status ifemgpu_learn_collect(ifemgpu_ctx* ctx, const double* rhs, const double* xstar,
                                     int stride, int max_iter, double rtol, int precond,
                                     int* pairs)
{
  ifemgpu_status st = deviceReady(ctx);
  if (st != IFEMGPU_OK) return st;
  if (!ctx->learn) return setError(ctx, IFEMGPU_NOT_READY, "learn_collect before learn_setup");
  if (!rhs && !ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "learn_collect before assemble");
  if (stride < 1 || max_iter < 1 || !(rtol > 0))
    return setError(ctx, IFEMGPU_INVALID_ARG, "learn_collect: bad stride, cap or tolerance");
  st = collectPairs(ctx, rhs, xstar, stride, max_iter, rtol, precond);
  if (pairs) *pairs = learnCount(ctx);
  return st;
}

ifemgpu_status ifemgpu_learn_clear(ifemgpu_ctx* ctx)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  learnClear(ctx);
  return IFEMGPU_OK;
}

ifemgpu_status ifemgpu_learn_set_target(ifemgpu_ctx* ctx, int mode)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  if (mode != IFEMGPU_LEARN_TARGET_ERROR && mode != IFEMGPU_LEARN_TARGET_COMPLEMENT)
    return setError(ctx, IFEMGPU_INVALID_ARG, "learn_set_target: unknown mode");
  return learnSetTarget(ctx, mode);
}

ifemgpu_status ifemgpu_learn_train(ifemgpu_ctx* ctx, int epochs, int batch, float lr,
                                   unsigned seed, float* final_loss)
{
  ifemgpu_status st = deviceReady(ctx);
  if (st != IFEMGPU_OK) return st;
  return learnTrain(ctx, epochs, batch, lr, seed, final_loss);
}

ifemgpu_status ifemgpu_learn_evaluate(ifemgpu_ctx* ctx, float* mse)
{
  ifemgpu_status st = deviceReady(ctx);
  if (st != IFEMGPU_OK) return st;
  return learnEvaluate(ctx, mse);
}

ifemgpu_status ifemgpu_learn_gradients(ifemgpu_ctx* ctx, const float* X, const float* Y, int n,
                                       float* grad, float* loss)
{
  ifemgpu_status st = deviceReady(ctx);
  if (st != IFEMGPU_OK) return st;
  return learnGradients(ctx, X, Y, n, grad, loss);
}

ifemgpu_status ifemgpu_learn_get_weights(ifemgpu_ctx* ctx, float* theta, int* count, float* scale)
{
  ifemgpu_status st = deviceReady(ctx);
  if (st != IFEMGPU_OK) return st;
  return learnWeights(ctx, theta, count, scale, 0);
}

ifemgpu_status ifemgpu_learn_set_weights(ifemgpu_ctx* ctx, const float* theta, int count,
                                         float scale)
{
  ifemgpu_status st = deviceReady(ctx);
  if (st != IFEMGPU_OK) return st;
  if (!theta) return setError(ctx, IFEMGPU_INVALID_ARG, "learn_set_weights: null array");
  return learnWeights(ctx, const_cast<float*>(theta), &count, &scale, 1);
}

ifemgpu_status ifemgpu_patch_update_field(ifemgpu_ctx* ctx, int patch_id, int which,
                                          const double* values)
{
  ifemgpu_status st = deviceReady(ctx);
  if (st != IFEMGPU_OK) return st;
  HostPatch* pc = getPatch(ctx, patch_id);
  if (!pc || !values) return setError(ctx, IFEMGPU_INVALID_ARG, "update_field: bad patch or values");
  std::vector<double>* host = nullptr;
  double* dev = nullptr;
  if (which == IFEMGPU_FIELD_LOG_KAPPA) { host = &pc->logk; dev = pc->d_logk; }
  else if (which == IFEMGPU_FIELD_SOURCE_NOISE) { host = &pc->noise; dev = pc->d_noise; }
  else return setError(ctx, IFEMGPU_INVALID_ARG, "update_field: unknown field");
  if (host->empty() || !dev)
    return setError(ctx, IFEMGPU_NOT_READY, "update_field: the field was not set before preprocess");
  std::copy(values, values + host->size(), host->begin());
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  IFEMGPU_CUDA(ctx, cudaMemcpy(dev, host->data(), sizeof(double) * host->size(), cudaMemcpyHostToDevice));
  ctx->assembled = false;
  ctx->fieldVersion++;
  return IFEMGPU_OK;
}

}  // extern "C"
