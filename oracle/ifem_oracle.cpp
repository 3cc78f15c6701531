// ifem_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU, FP64 restatement of IFEM's element integration + assembly path for
// structured spline patches.  It is the checker the GPU path is compared
// against and the timed CPU baseline ("port") of the benchmark.  Nothing in
// the product links, loads or calls this file.
//
// Every function names the IFEM source (path inside the IFEM tree, file:line)
// whose behaviour it restates.  Basis functions are not IFEM code (IFEM calls
// GoTools for them): they are computed with the published Cox-de Boor
// algorithms of Piegl & Tiller, "The NURBS Book", 2nd ed., A2.1 (FindSpan)
// and A2.3 (DersBasisFuns), and the rational quotient rule R = wN/W.
//
// Parity pins (checked by tests/test_oracle_golden.py against fixtures in
// tests/golden/ that were extracted from IFEM's own unit tests):
//   Gauss rules           src/Utility/Test/TestGaussQuadrature.C
//   SAM couplings/MEQN    src/LinAlg/Test/TestSAM.C + refdata/sam_2D_*_1P.ref
//   element operators     Apps/Utils/Test/TestEqualOrderOperators.C
//   Jacobian / dNdX       src/Utility/Test/TestCoordinateMapping.C:357-392
//   bilinear basis        src/Utility/Test/TestSplineUtils.C:98-162
//   MNPC                  src/ASM/Test/ASM3DTests.h:192-223
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kEpsZ = 1.0e-12;  // epsZ compile definition, CMakeLists.txt:535-540

// ---------------------------------------------------------------------------
// Gauss-Legendre rule on [-1,1], ascending abscissae (GaussQuadrature.C:18-212
// tabulates the same points).  Newton iteration on the Legendre polynomial.
void gaussLegendre(int n, double* xi, double* wt)
{
  for (int i = 0; i < (n + 1) / 2; i++) {
    double x = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= n; k++) {
        double pk = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      if (n == 1) { p1 = x; p0 = 1.0; }
      dp = n * (x * p1 - p0) / (x * x - 1.0);
      double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    double p0 = 1.0, p1 = x;
    for (int k = 2; k <= n; k++) {
      double pk = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = pk;
    }
    if (n == 1) { p1 = x; p0 = 1.0; }
    dp = n * (x * p1 - p0) / (x * x - 1.0);
    double w = 2.0 / ((1.0 - x * x) * dp * dp);
    xi[i] = -x;
    xi[n - 1 - i] = x;
    wt[i] = wt[n - 1 - i] = w;
  }
  if (n % 2 == 1) xi[n / 2] = 0.0;
}

// Piegl & Tiller A2.1: knot span index k with U[k] <= u < U[k+1].
int findSpan(int n, int p, double u, const double* U)
{
  if (u >= U[n]) return n - 1;
  if (u <= U[p]) {
    int k = p;
    while (k < n - 1 && U[k + 1] <= u) k++;
    return k;
  }
  int lo = p, hi = n;
  int mid = (lo + hi) / 2;
  while (u < U[mid] || u >= U[mid + 1]) {
    if (u < U[mid]) hi = mid; else lo = mid;
    mid = (lo + hi) / 2;
  }
  return mid;
}

// Piegl & Tiller A2.3: values and first nd derivatives of the p+1 non-zero
// B-spline basis functions on span k.  ders[(d)*(p+1)+j].
void dersBasisFuns(int k, double u, int p, int nd, const double* U, double* ders)
{
  double ndu[8][8], a[2][8], left[8], right[8];
  ndu[0][0] = 1.0;
  for (int j = 1; j <= p; j++) {
    left[j] = u - U[k + 1 - j];
    right[j] = U[k + j] - u;
    double saved = 0.0;
    for (int r = 0; r < j; r++) {
      ndu[j][r] = right[r + 1] + left[j - r];
      double temp = ndu[r][j - 1] / ndu[j][r];
      ndu[r][j] = saved + right[r + 1] * temp;
      saved = left[j - r] * temp;
    }
    ndu[j][j] = saved;
  }
  for (int j = 0; j <= p; j++) ders[j] = ndu[j][p];
  for (int r = 0; r <= p; r++) {
    int s1 = 0, s2 = 1;
    a[0][0] = 1.0;
    for (int kk = 1; kk <= nd; kk++) {
      double d = 0.0;
      int rk = r - kk, pk = p - kk;
      if (r >= kk) {
        a[s2][0] = a[s1][0] / ndu[pk + 1][rk];
        d = a[s2][0] * ndu[rk][pk];
      }
      int j1 = (rk >= -1) ? 1 : -rk;
      int j2 = (r - 1 <= pk) ? kk - 1 : p - r;
      for (int j = j1; j <= j2; j++) {
        a[s2][j] = (a[s1][j] - a[s1][j - 1]) / ndu[pk + 1][rk + j];
        d += a[s2][j] * ndu[rk + j][pk];
      }
      if (r <= pk) {
        a[s2][kk] = -a[s1][kk - 1] / ndu[pk + 1][r];
        d += a[s2][kk] * ndu[r][pk];
      }
      ders[kk * (p + 1) + r] = d;
      std::swap(s1, s2);
    }
  }
  int r = p;
  for (int kk = 1; kk <= nd; kk++) {
    for (int j = 0; j <= p; j++) ders[kk * (p + 1) + j] *= r;
    r *= (p - kk);
  }
}

struct Material {
  int kind = 0;  // 1 Poisson, 2 elasticity
  double kappa = 1.0, source = 0.0;
  int source_shape = 0;
  double E = 1.0, nu = 0.3;
  double body[3] = {0, 0, 0};
  double mass = 0.0;  // scale of the consistent mass matrix added to K
};

struct FaceBC { int face, dofs; double value; };
struct Connection { int master, mface, slave, sface, orient; };
struct Neumann { int face; double t[3]; };

struct Patch {
  int dim = 3;
  int p[3] = {0, 0, 0}, n[3] = {1, 1, 1};
  std::vector<double> U[3];
  std::vector<double> X;  // nnod x dim, Euclidean
  std::vector<double> W;  // nnod (1 if polynomial)
  bool rational = false;
  Material mat;
  int npv = 1;
  std::vector<double> logk, noise;
  std::vector<FaceBC> bcs;
  std::vector<Neumann> neumann;
  // topology
  int nel_d[3] = {1, 1, 1};
  int nnod = 0, nelAll = 0;
  std::vector<std::vector<int>> mnpc;  // per element (empty: zero span)
  std::vector<int> mlge;               // 0 for zero-span elements
  int firstNode = 0;                   // global node offset (0-based)
  std::vector<int> mlgn;               // global 0-based node per patch node
  int nen() const { return dim == 3 ? (p[0]+1)*(p[1]+1)*(p[2]+1) : (p[0]+1)*(p[1]+1); }
};

struct Model {
  std::vector<Patch> patches;
  std::vector<Connection> conns;
  int nGauss = 4;
  int nnod = 0, nel = 0, ndof = 0, neq = 0, nceq = 0;
  std::vector<int> madof, msc, meqn;
  std::vector<double> c0;  // prescribed value per constraint equation
  std::vector<int> mpmnpc, mmnpc;
  std::vector<int> IA, JA;
  std::vector<double> A, b;
  std::string err;
  bool bisect = false;  // entry lookup by binary search (parity tests of large models)
};

int numGauss(const Model& m, int order, bool neumann)
{
  // ASMbase::getNoGaussPt, src/ASM/ASMbase.C:1788-1798 (order = degree+1)
  int ng = m.nGauss;
  if (ng <= -order) return 0;
  if (ng > 0 && ng < 11) return ng;
  if (neumann) return order;
  return order + ng % 10;
}

// ASMs3D::generateFEMTopology (src/ASM/ASMs3D.C:487-509) and createMNPC
// (:3899-3924); ASMs2D counterparts (src/ASM/ASMs2D.C:501, :3342-3361).
void generateTopology(Patch& pc, int& gEl)
{
  const int d = pc.dim;
  pc.nnod = 1;
  for (int k = 0; k < d; k++) {
    pc.nel_d[k] = pc.n[k] - pc.p[k];
    pc.nnod *= pc.n[k];
  }
  if (d == 2) pc.nel_d[2] = 1, pc.n[2] = 1;
  pc.nelAll = pc.nel_d[0] * pc.nel_d[1] * pc.nel_d[2];
  pc.mnpc.assign(pc.nelAll, {});
  pc.mlge.assign(pc.nelAll, 0);
  const int n1 = pc.n[0], n2 = pc.n[1];
  const int q1 = pc.p[0], q2 = pc.p[1], q3 = d == 3 ? pc.p[2] : 0;
  int iel = 0;
  for (int e3 = 0; e3 < pc.nel_d[2]; e3++)
    for (int e2 = 0; e2 < pc.nel_d[1]; e2++)
      for (int e1 = 0; e1 < pc.nel_d[0]; e1++, iel++) {
        bool nz = pc.U[0][q1 + e1 + 1] > pc.U[0][q1 + e1] &&
                  pc.U[1][q2 + e2 + 1] > pc.U[1][q2 + e2] &&
                  (d == 2 || pc.U[2][q3 + e3 + 1] > pc.U[2][q3 + e3]);
        if (!nz) continue;
        pc.mlge[iel] = ++gEl;
        // last (highest) node of the element, then descending offsets
        int inod = ((e3 + q3) * n2 + (e2 + q2)) * n1 + e1 + q1;
        auto& v = pc.mnpc[iel];
        for (int j3 = q3; j3 >= 0; j3--)
          for (int j2 = q2; j2 >= 0; j2--)
            for (int j1 = q1; j1 >= 0; j1--)
              v.push_back(inod - n1 * n2 * j3 - n1 * j2 - j1);
      }
}

// Nodes of a face in the loop order of ASMs3D::constrainFace
// (src/ASM/ASMs3D.C:1044-1101) / ASMs2D::constrainEdge.
std::vector<int> faceNodes(const Patch& pc, int face)
{
  std::vector<int> out;
  const int n1 = pc.n[0], n2 = pc.n[1], n3 = pc.dim == 3 ? pc.n[2] : 1;
  int dir = (face + 1) / 2;          // 1,2,3
  bool hi = (face % 2) == 0;
  auto id = [&](int i, int j, int k) { return (k * n2 + j) * n1 + i; };
  if (dir == 1) {
    int i = hi ? n1 - 1 : 0;
    for (int k = 0; k < n3; k++)
      for (int j = 0; j < n2; j++) out.push_back(id(i, j, k));
  } else if (dir == 2) {
    int j = hi ? n2 - 1 : 0;
    for (int k = 0; k < n3; k++)
      for (int i = 0; i < n1; i++) out.push_back(id(i, j, k));
  } else {
    int k = hi ? n3 - 1 : 0;
    for (int j = 0; j < n2; j++)
      for (int i = 0; i < n1; i++) out.push_back(id(i, j, k));
  }
  return out;
}

// SAMpatch::init -> initNodeDofs / initElementConn / initConstraintEqs and
// SAM::initSystemEquations (src/ASM/SAMpatch.C:21-360, src/LinAlg/SAM.C:225-336),
// restricted to fixed and prescribed (master-less) constraints.
// Patch connections: ASMs3D::connectPatch / connectBasis and
// ASMs2D::connectBasis (src/ASM/ASMs3D.C:700-796, ASMs2D.C:697-749) with
// ASMbase::collapseNodes / mergeNodes (src/ASM/ASMbase.C:1289-1331): the
// slave face's nodes, in the master face's node order under orientation
// `orient`, take the smaller of the two global numbers, a change reaching
// the patches already connected to the changed one.  Then
// SIMbase::renumberNodes (src/SIM/SIMbase.C:535-565): numbers compacted in
// order of first appearance.  G holds 1-based numbers; returns the count,
// or -1 when faces do not match.
int connectPatches(Model& m, std::vector<std::vector<int>>& G)
{
  const size_t np = m.patches.size();
  std::vector<std::vector<int>> nb(np);
  auto faceDims = [](const Patch& pc, int face, int& a, int& b) {
    const int dir = (face + 1) / 2;
    if (pc.dim == 2) { a = dir == 1 ? pc.n[1] : pc.n[0]; b = 1; }
    else if (dir == 1) { a = pc.n[1]; b = pc.n[2]; }
    else if (dir == 2) { a = pc.n[0]; b = pc.n[2]; }
    else { a = pc.n[0]; b = pc.n[1]; }
  };
  for (const Connection& c : m.conns) {
    const int M = c.master - 1, S = c.slave - 1;
    const Patch &pm = m.patches[M], &ps = m.patches[S];
    const std::vector<int> mn = faceNodes(pm, c.mface), sn = faceNodes(ps, c.sface);
    int m1, m2, n1, n2;
    faceDims(ps, c.sface, m1, m2);
    faceDims(pm, c.mface, n1, n2);
    const bool swapped = pm.dim == 3 && c.orient > 3;
    if ((swapped ? n2 : n1) != m1 || (swapped ? n1 : n2) != m2) return -1;
    int node = 0;
    for (int j = 0; j < n2; j++)
      for (int i = 0; i < n1; i++, node++) {
        int k = i, l = j;
        if (pm.dim == 3) {
          const int o = c.orient;
          if (o & 4) { k = j; l = i; }
          if (o == 1 || o == 3) l = n2 - 1 - j;
          if (o == 2 || o == 3) k = n1 - 1 - i;
          if (o == 5 || o == 7) l = m2 - 1 - i;
          if (o == 6 || o == 7) k = m1 - 1 - j;
        } else if (c.orient) {
          k = n1 - 1 - i;
        }
        const int snode = sn[(size_t)l * m1 + k], mnode = mn[node];
        for (int d = 0; d < pm.dim; d++)
          if (std::fabs(pm.X[(size_t)mnode * pm.dim + d] - ps.X[(size_t)snode * ps.dim + d]) > 1e-4)
            return -1;
        int& gm = G[M][mnode];
        int& gs = G[S][snode];
        if (gm == gs) continue;
        const int P = gm > gs ? M : S, inod = gm > gs ? mnode : snode;
        const int oldNum = G[P][inod], newNum = std::min(gm, gs);
        G[P][inod] = newNum;
        for (int Q : nb[P])
          for (int& g : G[Q])
            if (g == oldNum) g = newNum;
      }
    if (std::find(nb[S].begin(), nb[S].end(), M) == nb[S].end()) {
      nb[S].push_back(M);
      nb[M].push_back(S);
    }
  }
  std::map<int, int> renum;
  int count = 0;
  for (size_t P = 0; P < np; P++) {
    bool changed = false;
    for (int& g : G[P]) {
      auto it = renum.find(g);
      if (it == renum.end()) it = renum.emplace(g, ++count).first;
      if (it->second != g) {
        g = it->second;
        changed = true;
      }
    }
    if (!changed && !G[P].empty()) count = std::max(count, *std::max_element(G[P].begin(), G[P].end()));
  }
  return count;
}

bool initSAM(Model& m)
{
  int gEl = 0, gNod = 0;
  for (auto& pc : m.patches) {
    generateTopology(pc, gEl);
    pc.firstNode = gNod;
    gNod += pc.nnod;
  }
  std::vector<std::vector<int>> G(m.patches.size());
  for (size_t p = 0; p < m.patches.size(); p++)
    for (int i = 0; i < m.patches[p].nnod; i++) G[p].push_back(m.patches[p].firstNode + i + 1);
  if (!m.conns.empty() && (gNod = connectPatches(m, G)) < 0) {
    m.err = "non-matching patch connection";
    return false;
  }
  for (size_t p = 0; p < m.patches.size(); p++) {
    m.patches[p].mlgn = G[p];
    for (int& g : m.patches[p].mlgn) g -= 1;
  }
  m.nnod = gNod;
  m.nel = gEl;
  m.madof.assign(m.nnod + 1, 0);
  for (auto& pc : m.patches)
    for (int i = 0; i < pc.nnod; i++) m.madof[pc.mlgn[i] + 1] = pc.npv;
  m.madof[0] = 1;
  for (int i = 0; i < m.nnod; i++) m.madof[i + 1] += m.madof[i];
  m.ndof = m.madof[m.nnod] - 1;
  m.msc.assign(m.ndof, 1);
  std::vector<int> slaveOf(m.ndof, 0);  // constraint index (1-based) per DOF
  m.c0.clear();
  // homogeneous constraints first set the status codes (BC codes CX..RZ)
  for (auto& pc : m.patches)
    for (auto& bc : pc.bcs) {
      if (bc.value != 0.0) continue;
      for (int node : faceNodes(pc, bc.face))
        for (char c : std::to_string(bc.dofs)) {
          int dof = c - '0';
          if (dof < 1 || dof > pc.npv) continue;
          m.msc[m.madof[pc.mlgn[node]] - 1 + dof - 1] = 0;
        }
    }
  // prescribed DOFs: one constraint equation each, first one wins, fixed wins
  for (auto& pc : m.patches)
    for (auto& bc : pc.bcs) {
      if (bc.value == 0.0) continue;
      for (int node : faceNodes(pc, bc.face))
        for (char c : std::to_string(bc.dofs)) {
          int dof = c - '0';
          if (dof < 1 || dof > pc.npv) continue;
          int idof = m.madof[pc.mlgn[node]] - 1 + dof - 1;
          if (m.msc[idof] <= 0 || slaveOf[idof]) continue;
          m.c0.push_back(bc.value);
          slaveOf[idof] = (int)m.c0.size();
        }
    }
  m.nceq = (int)m.c0.size();
  m.meqn.assign(m.ndof, 0);
  for (int i = 0; i < m.ndof; i++)
    if (slaveOf[i]) { m.meqn[i] = -slaveOf[i]; m.msc[i] = 0; }
  int ieq = 0;
  for (int i = 0; i < m.ndof; i++)
    if (m.msc[i] == 1) m.meqn[i] = ++ieq;
  m.neq = ieq;
  // element connectivity MPMNPC/MMNPC (1-based global nodes)
  m.mpmnpc.assign(1, 1);
  m.mmnpc.clear();
  for (auto& pc : m.patches)
    for (int e = 0; e < pc.nelAll; e++)
      if (pc.mlge[e] > 0) {
        for (int nd : pc.mnpc[e]) m.mmnpc.push_back(pc.mlgn[nd] + 1);
        m.mpmnpc.push_back((int)m.mmnpc.size() + 1);
      }
  return true;
}

// SAM::getElmEqns, src/LinAlg/SAM.C:655-696 (iel 1-based)
void getElmEqns(const Model& m, int iel, std::vector<int>& meen)
{
  meen.clear();
  for (int ip = m.mpmnpc[iel - 1]; ip < m.mpmnpc[iel]; ip++) {
    int node = m.mmnpc[ip - 1];
    for (int d = m.madof[node - 1]; d < m.madof[node]; d++)
      meen.push_back(m.meqn[d - 1]);
  }
}

// SAM::getDofCouplings (src/LinAlg/SAM.C:377-427, no master DOFs) and
// SparseMatrix::optimiseCols(dofc) (src/LinAlg/SparseMatrix.C:984-1023).
void buildPattern(Model& m)
{
  std::vector<std::set<int>> dofc(m.neq);
  std::vector<int> meen;
  for (int iel = 1; iel <= m.nel; iel++) {
    getElmEqns(m, iel, meen);
    for (size_t j = 0; j < meen.size(); j++) {
      int jeq = meen[j];
      if (jeq <= 0) continue;
      dofc[jeq - 1].insert(jeq);
      for (size_t i = 0; i < j; i++) {
        int ieq = meen[i];
        if (ieq > 0) {
          dofc[ieq - 1].insert(jeq);
          dofc[jeq - 1].insert(ieq);
        }
      }
    }
  }
  m.IA.assign(m.neq + 1, 0);
  size_t nnz = 0;
  for (int i = 0; i < m.neq; i++) {
    nnz += dofc[i].size();
    for (int k : dofc[i]) m.IA[k - 1]++;
  }
  int k = 0, jsize = m.IA[0];
  m.IA[0] = 0;
  for (int j = 1; j < m.neq; j++) {
    k += jsize;
    jsize = m.IA[j];
    m.IA[j] = k;
  }
  m.JA.assign(nnz, 0);
  for (int i = 0; i < m.neq; i++)
    for (int kk : dofc[i]) m.JA[m.IA[kk - 1]++] = i;
  for (int j = m.neq; j > 0; j--) m.IA[j] = m.IA[j - 1];
  m.IA[0] = 0;
  m.A.assign(nnz, 0.0);
  m.b.assign(m.neq, 0.0);
}

// The same compressed-column pattern as buildPattern for large models (the
// std::set couplings of SAM::getDofCouplings take minutes and tens of GB at
// 3e8 entries): all DOFs of a node couple with the same equations -- the free
// DOFs of every node that shares an element with it -- and equations grow
// with the global node number (node-major DOFs, free DOFs numbered in DOF
// order), so a node's sorted, de-duplicated neighbour nodes give each of its
// columns in ascending row order.  Nodes are processed in parallel.
void buildPatternFast(Model& m)
{
  // elements around each global node (0-based nodes, 1-based elements)
  std::vector<int> start(m.nnod + 1, 0);
  for (int iel = 1; iel <= m.nel; iel++)
    for (int ip = m.mpmnpc[iel - 1]; ip < m.mpmnpc[iel]; ip++) start[m.mmnpc[ip - 1]]++;
  for (int n = 0; n < m.nnod; n++) start[n + 1] += start[n];
  std::vector<int> elms(start[m.nnod]);
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int iel = 1; iel <= m.nel; iel++)
      for (int ip = m.mpmnpc[iel - 1]; ip < m.mpmnpc[iel]; ip++)
        elms[fill[m.mmnpc[ip - 1] - 1]++] = iel;
  }
  auto freeEqs = [&](int node, std::vector<int>& out) {  // node 0-based
    for (int d = m.madof[node]; d < m.madof[node + 1]; d++)
      if (m.meqn[d - 1] > 0) out.push_back(m.meqn[d - 1]);
  };
  auto neighbours = [&](int node, std::vector<int>& nb) {
    nb.clear();
    for (int k = start[node]; k < start[node + 1]; k++) {
      const int iel = elms[k];
      for (int ip = m.mpmnpc[iel - 1]; ip < m.mpmnpc[iel]; ip++) nb.push_back(m.mmnpc[ip - 1] - 1);
    }
    std::sort(nb.begin(), nb.end());
    nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
  };
  // column lengths, then the row indices
  std::vector<long long> len(m.nnod, 0);
#pragma omp parallel
  {
    std::vector<int> nb, eqs;
#pragma omp for schedule(dynamic, 256)
    for (int n = 0; n < m.nnod; n++) {
      neighbours(n, nb);
      eqs.clear();
      for (int b : nb) freeEqs(b, eqs);
      len[n] = (long long)eqs.size();
    }
  }
  m.IA.assign(m.neq + 1, 0);
  std::vector<int> own;
  for (int n = 0; n < m.nnod; n++) {
    own.clear();
    freeEqs(n, own);
    for (int q : own) m.IA[q] = (int)len[n];
  }
  for (int j = 0; j < m.neq; j++) m.IA[j + 1] += m.IA[j];
  m.JA.assign(m.IA[m.neq], 0);
#pragma omp parallel
  {
    std::vector<int> nb, eqs, mine;
#pragma omp for schedule(dynamic, 256)
    for (int n = 0; n < m.nnod; n++) {
      mine.clear();
      freeEqs(n, mine);
      if (mine.empty()) continue;
      neighbours(n, nb);
      eqs.clear();
      for (int b : nb) freeEqs(b, eqs);
      for (int q : mine)
        for (size_t i = 0; i < eqs.size(); i++) m.JA[m.IA[q - 1] + i] = eqs[i] - 1;
    }
  }
  m.A.assign(m.JA.size(), 0.0);
  m.b.assign(m.neq, 0.0);
}

// SparseMatrix::operator() compressed-column branch, SparseMatrix.C:283-289
// (a linear std::find over the column's rows).  m.bisect replaces the linear
// search by a binary search over the same ascending rows (same entry, same
// sums; only the parity tests of large models use it, never the timed
// baseline).
inline double& entry(Model& m, int r, int c)
{
  auto b = m.JA.begin() + m.IA[c - 1], e = m.JA.begin() + m.IA[c];
  auto it = m.bisect ? std::lower_bound(b, e, r - 1) : std::find(b, e, r - 1);
  if (it != e && *it != r - 1) it = e;
  static double dummy;
  if (it == e) { dummy = 0; return dummy; }
  return m.A[it - m.JA.begin()];
}

// assemSparse (src/LinAlg/SparseMatrix.C:614-688) for fixed and prescribed
// DOFs, preceded by the element RHS vector (SAM::assembleSystem(b,eS,iel) ->
// assembleRHS, src/LinAlg/SAM.C:518-543, :605-617) as AlgEqSystem::assemble
// orders them (src/ASM/AlgEqSystem.C:229-243).  eK is column-major.
void assembleElement(Model& m, int iel, const std::vector<double>& eK,
                     const std::vector<double>& eS, std::vector<int>& meen)
{
  getElmEqns(m, iel, meen);
  const int nedof = (int)meen.size();
  for (int i = 0; i < nedof; i++)
    if (meen[i] > 0) m.b[meen[i] - 1] += eS[i];
  auto K = [&](int i, int j) { return eK[(size_t)j * nedof + i]; };
  for (int j = 1; j <= nedof; j++) {
    int jeq = meen[j - 1];
    if (jeq < 1) continue;
    entry(m, jeq, jeq) += K(j - 1, j - 1);
    for (int i = 1; i < j; i++) {
      int ieq = meen[i - 1];
      if (ieq < 1) continue;
      entry(m, ieq, jeq) += K(i - 1, j - 1);
      entry(m, jeq, ieq) += K(j - 1, i - 1);
    }
  }
  for (int j = 1; j <= nedof; j++) {
    int jceq = -meen[j - 1];
    if (jceq < 1) continue;
    double c0 = m.c0[jceq - 1];
    for (int i = 1; i <= nedof; i++) {
      int ieq = meen[i - 1];
      if (ieq > 0) m.b[ieq - 1] -= c0 * K(i - 1, j - 1);
    }
  }
}

// Element-local evaluation of the rational basis at one integration point:
// N (nen), dNdu (nen x dim, column-major), from the 1D B-spline factors.
struct Basis1D { double N[8], dN[8]; };

void eval1D(const Patch& pc, int d, int span, double u, Basis1D& out)
{
  double ders[2 * 8];
  dersBasisFuns(span, u, pc.p[d], 1, pc.U[d].data(), ders);
  for (int j = 0; j <= pc.p[d]; j++) {
    out.N[j] = ders[j];
    out.dN[j] = ders[pc.p[d] + 1 + j];
  }
}

void tensorBasis(const Patch& pc, const Basis1D* b, const std::vector<int>& nodes,
                 std::vector<double>& N, std::vector<double>& dNdu)
{
  const int dim = pc.dim, nen = (int)nodes.size();
  const int q1 = pc.p[0] + 1, q2 = pc.p[1] + 1;
  N.assign(nen, 0.0);
  dNdu.assign((size_t)nen * dim, 0.0);
  for (int a = 0; a < nen; a++) {
    int i = a % q1, j = (a / q1) % q2, k = a / (q1 * q2);
    if (dim == 2) {
      N[a] = b[0].N[i] * b[1].N[j];
      dNdu[a] = b[0].dN[i] * b[1].N[j];
      dNdu[nen + a] = b[0].N[i] * b[1].dN[j];
    } else {
      N[a] = b[0].N[i] * b[1].N[j] * b[2].N[k];
      dNdu[a] = b[0].dN[i] * b[1].N[j] * b[2].N[k];
      dNdu[nen + a] = b[0].N[i] * b[1].dN[j] * b[2].N[k];
      dNdu[2 * nen + a] = b[0].N[i] * b[1].N[j] * b[2].dN[k];
    }
  }
  if (!pc.rational) return;
  double Wt = 0.0, dW[3] = {0, 0, 0};
  for (int a = 0; a < nen; a++) {
    double w = pc.W[nodes[a]];
    Wt += w * N[a];
    for (int c = 0; c < dim; c++) dW[c] += w * dNdu[(size_t)c * nen + a];
  }
  for (int a = 0; a < nen; a++) {
    double w = pc.W[nodes[a]];
    double R = w * N[a] / Wt;
    for (int c = 0; c < dim; c++)
      dNdu[(size_t)c * nen + a] = (w * dNdu[(size_t)c * nen + a] - R * dW[c]) / Wt;
    N[a] = R;
  }
}

// utl::Jacobian (src/Utility/CoordinateMapping.C:24-63) with
// matrix::inverse/det (src/LinAlg/matrix.h:790-850).  J (dim x dim,
// column-major) = X * dNdu; returns det J (0 if |det| <= epsZ) and dNdX.
double jacobian(int dim, int nen, const double* Xn, const double* dNdu,
                double* Jout, double* dNdX)
{
  double J[9] = {0};
  for (int r = 0; r < dim; r++)
    for (int c = 0; c < dim; c++) {
      double s = 0.0;
      for (int a = 0; a < nen; a++) s += Xn[(size_t)a * dim + r] * dNdu[(size_t)c * nen + a];
      J[c * dim + r] = s;
    }
  auto T = [&](int i, int j) { return J[(j - 1) * dim + (i - 1)]; };
  double det, B[9];
  if (dim == 2) {
    det = T(1, 1) * T(2, 2) - T(2, 1) * T(1, 2);
    if (det <= kEpsZ && det >= -kEpsZ) return 0.0;
    B[0] = T(2, 2) / det; B[1] = -T(2, 1) / det;
    B[2] = -T(1, 2) / det; B[3] = T(1, 1) / det;
  } else {
    det = T(1, 1) * (T(2, 2) * T(3, 3) - T(3, 2) * T(2, 3))
        - T(1, 2) * (T(2, 1) * T(3, 3) - T(3, 1) * T(2, 3))
        + T(1, 3) * (T(2, 1) * T(3, 2) - T(3, 1) * T(2, 2));
    if (det <= kEpsZ && det >= -kEpsZ) return 0.0;
    B[0] =  (T(2, 2) * T(3, 3) - T(3, 2) * T(2, 3)) / det;
    B[1] = -(T(2, 1) * T(3, 3) - T(3, 1) * T(2, 3)) / det;
    B[2] =  (T(2, 1) * T(3, 2) - T(3, 1) * T(2, 2)) / det;
    B[3] = -(T(1, 2) * T(3, 3) - T(3, 2) * T(1, 3)) / det;
    B[4] =  (T(1, 1) * T(3, 3) - T(3, 1) * T(1, 3)) / det;
    B[5] = -(T(1, 1) * T(3, 2) - T(3, 1) * T(1, 2)) / det;
    B[6] =  (T(1, 2) * T(2, 3) - T(2, 2) * T(1, 3)) / det;
    B[7] = -(T(1, 1) * T(2, 3) - T(2, 1) * T(1, 3)) / det;
    B[8] =  (T(1, 1) * T(2, 2) - T(2, 1) * T(1, 2)) / det;
  }
  if (Jout) std::memcpy(Jout, J, sizeof(double) * dim * dim);
  // dNdX = dNdu * J^-1  (B holds J^-1 column-major)
  for (int a = 0; a < nen; a++)
    for (int c = 0; c < dim; c++) {
      double s = 0.0;
      for (int k = 0; k < dim; k++) s += dNdu[(size_t)k * nen + a] * B[c * dim + k];
      dNdX[(size_t)c * nen + a] = s;
    }
  return det;
}

// Face Jacobian: utl::Jacobian(J,n,dNdX,X,dNdu,t1,t2) (CoordinateMapping.C:90-133)
double faceJacobian(int nen, const double* Xn, const double* dNdu, int t1, int t2,
                    double* normal)
{
  double J[9] = {0};
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      double s = 0.0;
      for (int a = 0; a < nen; a++) s += Xn[(size_t)a * 3 + r] * dNdu[(size_t)c * nen + a];
      J[c * 3 + r] = s;
    }
  const double* a = J + 3 * (t1 - 1);
  const double* b = J + 3 * (t2 - 1);
  double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  double dS = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  for (int i = 0; i < 3; i++) normal[i] = dS > 0 ? n[i] / dS : 0.0;
  double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[3] * (J[1] * J[8] - J[2] * J[7])
             + J[6] * (J[1] * J[5] - J[2] * J[4]);
  if (det <= kEpsZ && det >= -kEpsZ) return 0.0;
  return dS;
}

// Weak forms.  Poisson: EqualOrderOperators::Weak::LaplacianCoeff (scalar
// kappa) and Source (Apps/Utils/EqualOrderOperators.C:194-211, :243-265).
// Elasticity: Ke += B^T (D B) detJxW with the 6 x (3 nen) strain matrix of
// node-interleaved DOFs, the formulation of IFEM's linear-elasticity
// integrands; restated here from the textbook isotropic constitutive law.
struct Scratch {
  std::vector<double> N, dNdu, dNdX, Bm, DB;
};

void evalPoisson(const Patch& pc, int nen, double detJxW, const std::vector<double>& N,
                 const std::vector<double>& dNdX, const double* X,
                 const std::vector<int>& nodes, std::vector<double>& eK,
                 std::vector<double>& eS)
{
  const int dim = pc.dim;
  double kap = pc.mat.kappa;
  if (!pc.logk.empty()) {
    double g = 0.0;
    for (int a = 0; a < nen; a++) g += N[a] * pc.logk[nodes[a]];
    kap *= std::exp(g);
  }
  double s = kap * detJxW;
  // EM += (grad*s) * grad^T  (matrix<T>::multiply with addTo)
  for (int j = 0; j < nen; j++)
    for (int i = 0; i < nen; i++) {
      double v = 0.0;
      for (int c = 0; c < dim; c++) v += dNdX[(size_t)c * nen + i] * s * dNdX[(size_t)c * nen + j];
      eK[(size_t)j * nen + i] += v;
    }
  // EqualOrderOperators::Weak::Mass (Apps/Utils/EqualOrderOperators.C:214-227)
  if (pc.mat.mass != 0.0)
    for (int j = 0; j < nen; j++)
      for (int i = 0; i < nen; i++) eK[(size_t)j * nen + i] += N[i] * N[j] * pc.mat.mass * detJxW;
  if (pc.mat.source != 0.0) {
    double f = pc.mat.source;
    if (pc.mat.source_shape == 1)
      for (int c = 0; c < dim; c++) f *= std::sin(M_PI * X[c]);
    if (!pc.noise.empty()) {
      double e = 0.0;
      for (int a = 0; a < nen; a++) e += N[a] * pc.noise[nodes[a]];
      f *= 1.0 + e;
    }
    for (int a = 0; a < nen; a++) eS[a] += N[a] * f * detJxW;
  }
}

void evalElasticity(const Patch& pc, int nen, double detJxW, const std::vector<double>& N,
                    const std::vector<double>& dNdX, Scratch& s,
                    std::vector<double>& eK, std::vector<double>& eS)
{
  const int nd = 3 * nen;
  const double E = pc.mat.E, nu = pc.mat.nu;
  const double lam = E * nu / ((1 + nu) * (1 - 2 * nu)), mu = E / (2 * (1 + nu));
  double D[36] = {0};
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) D[j * 6 + i] = lam;
    D[i * 6 + i] = lam + 2 * mu;
    D[(i + 3) * 6 + i + 3] = mu;
  }
  // B (6 x nd, column-major): rows exx eyy ezz gxy gyz gzx
  s.Bm.assign((size_t)6 * nd, 0.0);
  auto B = [&](int r, int c) -> double& { return s.Bm[(size_t)c * 6 + r]; };
  for (int a = 0; a < nen; a++) {
    double dx = dNdX[a], dy = dNdX[nen + a], dz = dNdX[2 * nen + a];
    B(0, 3 * a) = dx;
    B(1, 3 * a + 1) = dy;
    B(2, 3 * a + 2) = dz;
    B(3, 3 * a) = dy; B(3, 3 * a + 1) = dx;
    B(4, 3 * a + 1) = dz; B(4, 3 * a + 2) = dy;
    B(5, 3 * a) = dz; B(5, 3 * a + 2) = dx;
  }
  // DB = D * B * detJxW ; EM += B^T * DB
  s.DB.assign((size_t)6 * nd, 0.0);
  for (int c = 0; c < nd; c++)
    for (int r = 0; r < 6; r++) {
      double v = 0.0;
      for (int k = 0; k < 6; k++) v += D[k * 6 + r] * s.Bm[(size_t)c * 6 + k];
      s.DB[(size_t)c * 6 + r] = v * detJxW;
    }
  for (int j = 0; j < nd; j++)
    for (int i = 0; i < nd; i++) {
      double v = 0.0;
      for (int k = 0; k < 6; k++) v += s.Bm[(size_t)i * 6 + k] * s.DB[(size_t)j * 6 + k];
      eK[(size_t)j * nd + i] += v;
    }
  if (pc.mat.mass != 0.0)  // Weak::Mass per component (EqualOrderOperators.C:214-227)
    for (int b = 0; b < nen; b++)
      for (int a = 0; a < nen; a++)
        for (int c = 0; c < 3; c++)
          eK[(size_t)(3 * b + c) * nd + 3 * a + c] += N[a] * N[b] * pc.mat.mass * detJxW;
  for (int a = 0; a < nen; a++)
    for (int c = 0; c < 3; c++) eS[3 * a + c] += pc.mat.body[c] * N[a] * detJxW;
}

// Gauss parameters of span e: SplineUtils::getGaussParameters (SplineUtils.C:200-220)
inline double gaussParam(const Patch& pc, int d, int e, double xi)
{
  double u0 = pc.U[d][pc.p[d] + e], u1 = pc.U[d][pc.p[d] + e + 1];
  return 0.5 * ((u1 - u0) * xi + u1 + u0);
}

// Element loop body of ASMs3D::integrate (src/ASM/ASMs3D.C:2128-2325) and
// ASMs2D::integrate (src/ASM/ASMs2D.C:1718-1991).
int integrateElement(Model& m, Patch& pc, int iel, const int ng[3],
                     const double* xg[3], const double* wg[3], Scratch& s,
                     std::vector<double>& eK, std::vector<double>& eS,
                     std::vector<int>& meen, bool doAssemble)
{
  const int dim = pc.dim, nen = pc.nen();
  const auto& nodes = pc.mnpc[iel];
  if (nodes.empty()) return 0;
  const int e1 = iel % pc.nel_d[0], e2 = (iel / pc.nel_d[0]) % pc.nel_d[1];
  const int e3 = iel / (pc.nel_d[0] * pc.nel_d[1]);
  const int ee[3] = {e1, e2, e3};
  double dV = dim == 3 ? 0.125 : 0.25;
  for (int d = 0; d < dim; d++)
    dV *= pc.U[d][pc.p[d] + ee[d] + 1] - pc.U[d][pc.p[d] + ee[d]];
  std::vector<double> Xn((size_t)nen * dim);
  for (int a = 0; a < nen; a++)
    for (int c = 0; c < dim; c++) Xn[(size_t)a * dim + c] = pc.X[(size_t)nodes[a] * dim + c];
  const int nd = nen * pc.npv;
  eK.assign((size_t)nd * nd, 0.0);
  eS.assign(nd, 0.0);
  s.dNdX.assign((size_t)nen * dim, 0.0);
  int singular = 0;
  Basis1D b[3];
  const int ng3 = dim == 3 ? ng[2] : 1;
  for (int k = 0; k < ng3; k++)
    for (int j = 0; j < ng[1]; j++)
      for (int i = 0; i < ng[0]; i++) {
        const int gi[3] = {i, j, k};
        for (int d = 0; d < dim; d++) {
          double u = gaussParam(pc, d, ee[d], xg[d][gi[d]]);
          eval1D(pc, d, pc.p[d] + ee[d], u, b[d]);
        }
        tensorBasis(pc, b, nodes, s.N, s.dNdu);
        double det = jacobian(dim, nen, Xn.data(), s.dNdu.data(), nullptr, s.dNdX.data());
        if (det == 0.0) { singular++; continue; }
        double X[3] = {0, 0, 0};
        for (int a = 0; a < nen; a++)
          for (int c = 0; c < dim; c++) X[c] += Xn[(size_t)a * dim + c] * s.N[a];
        double detJxW = det * dV * wg[0][i] * wg[1][j] * (dim == 3 ? wg[2][k] : 1.0);
        if (pc.mat.kind == 1)
          evalPoisson(pc, nen, detJxW, s.N, s.dNdX, X, nodes, eK, eS);
        else
          evalElasticity(pc, nen, detJxW, s.N, s.dNdX, s, eK, eS);
      }
  if (doAssemble) assembleElement(m, pc.mlge[iel], eK, eS, meen);
  return singular;
}

// Energy and L2 norms of a DOF-order field u over one element, and the
// secondary solution (Poisson flux -kappa grad u, elasticity stress in
// Voigt order xx yy zz xy yz zx) at its Gauss points: the norm integrands
// of the Poisson and elasticity applications as SIMbase::solutionNorms
// (src/SIM/SIMbase.C:1838-1967) integrates them, and the point evaluation
// of ASMs3D::evalSolution (src/ASM/ASMs3D.C:3179-3500) at the Gauss points.
void elementNorms(const Model& m, Patch& pc, int iel, const double* u, double out[2],
                  double* sec)
{
  out[0] = out[1] = 0.0;
  const int dim = pc.dim, nen = pc.nen(), npv = pc.npv;
  const auto& nodes = pc.mnpc[iel];
  if (nodes.empty()) return;
  int ng[3] = {1, 1, 1};
  std::vector<double> xg[3], wg[3];
  for (int d = 0; d < dim; d++) {
    ng[d] = numGauss(m, pc.p[d] + 1, false);
    xg[d].resize(ng[d]);
    wg[d].resize(ng[d]);
    gaussLegendre(ng[d], xg[d].data(), wg[d].data());
  }
  const int ee[3] = {iel % pc.nel_d[0], (iel / pc.nel_d[0]) % pc.nel_d[1],
                     iel / (pc.nel_d[0] * pc.nel_d[1])};
  double dV = dim == 3 ? 0.125 : 0.25;
  for (int d = 0; d < dim; d++) dV *= pc.U[d][pc.p[d] + ee[d] + 1] - pc.U[d][pc.p[d] + ee[d]];
  std::vector<double> Xn((size_t)nen * dim), Ue((size_t)nen * 3, 0.0);
  for (int a = 0; a < nen; a++) {
    for (int c = 0; c < dim; c++) Xn[(size_t)a * dim + c] = pc.X[(size_t)nodes[a] * dim + c];
    const int d0 = m.madof[pc.mlgn[nodes[a]]] - 1;
    for (int c = 0; c < npv; c++) Ue[(size_t)a * 3 + c] = u[d0 + c];
  }
  const double E = pc.mat.E, nu = pc.mat.nu;
  const double lam = E * nu / ((1 + nu) * (1 - 2 * nu)), mu = E / (2 * (1 + nu));
  const int nc = pc.mat.kind == 1 ? dim : 6;
  std::vector<double> N, dNdu, dNdX((size_t)nen * dim);
  Basis1D b[3];
  int q = 0;
  for (int k = 0; k < (dim == 3 ? ng[2] : 1); k++)
    for (int j = 0; j < ng[1]; j++)
      for (int i = 0; i < ng[0]; i++, q++) {
        const int gi[3] = {i, j, k};
        for (int d = 0; d < dim; d++)
          eval1D(pc, d, pc.p[d] + ee[d], gaussParam(pc, d, ee[d], xg[d][gi[d]]), b[d]);
        tensorBasis(pc, b, nodes, N, dNdu);
        const double det = jacobian(dim, nen, Xn.data(), dNdu.data(), nullptr, dNdX.data());
        if (det == 0.0) continue;
        const double w = det * dV * wg[0][i] * wg[1][j] * (dim == 3 ? wg[2][k] : 1.0);
        double uh[3] = {0, 0, 0}, g[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, lk = 0.0;
        for (int a = 0; a < nen; a++) {
          for (int c = 0; c < npv; c++) {
            uh[c] += N[a] * Ue[(size_t)a * 3 + c];
            for (int r = 0; r < dim; r++) g[c][r] += dNdX[(size_t)r * nen + a] * Ue[(size_t)a * 3 + c];
          }
          if (!pc.logk.empty()) lk += N[a] * pc.logk[nodes[a]];
        }
        double energy, sv[6] = {0, 0, 0, 0, 0, 0};
        if (pc.mat.kind == 1) {
          const double kap = pc.mat.kappa * (pc.logk.empty() ? 1.0 : std::exp(lk));
          energy = kap * (g[0][0] * g[0][0] + g[0][1] * g[0][1] + g[0][2] * g[0][2]);
          for (int r = 0; r < dim; r++) sv[r] = -kap * g[0][r];
        } else {
          const double exx = g[0][0], eyy = g[1][1], ezz = g[2][2];
          const double gxy = g[0][1] + g[1][0], gyz = g[1][2] + g[2][1], gzx = g[2][0] + g[0][2];
          const double tr = exx + eyy + ezz;
          sv[0] = lam * tr + 2 * mu * exx;
          sv[1] = lam * tr + 2 * mu * eyy;
          sv[2] = lam * tr + 2 * mu * ezz;
          sv[3] = mu * gxy;
          sv[4] = mu * gyz;
          sv[5] = mu * gzx;
          energy = sv[0] * exx + sv[1] * eyy + sv[2] * ezz + sv[3] * gxy + sv[4] * gyz + sv[5] * gzx;
        }
        double l2 = 0.0;
        for (int c = 0; c < npv; c++) l2 += uh[c] * uh[c];
        out[0] += w * energy;
        out[1] += w * l2;
        if (sec)
          for (int c = 0; c < nc; c++) sec[(size_t)q * nc + c] = sv[c];
      }
}

// Face overload of ASMs3D::integrate (src/ASM/ASMs3D.C:2547-2812) for
// constant tractions (elasticity) or normal flux (Poisson).
void integrateNeumann(Model& m, Patch& pc, const Neumann& nm)
{
  if (pc.dim != 3) return;
  const int face = nm.face;
  const int faceDir = (face % 10 + 1) / ((face % 2) ? -2 : 2);
  const int t1 = 1 + std::abs(faceDir) % 3, t2 = 1 + t1 % 3;
  const int nd0 = std::abs(faceDir) - 1;
  int ng[3];
  std::vector<double> xg[3], wg[3];
  for (int d = 0; d < 3; d++) {
    if (d == nd0) { ng[d] = 1; continue; }
    ng[d] = numGauss(m, pc.p[d] + 1, true);
    xg[d].resize(ng[d]);
    wg[d].resize(ng[d]);
    gaussLegendre(ng[d], xg[d].data(), wg[d].data());
  }
  const int nen = pc.nen(), npv = pc.npv;
  Scratch s;
  std::vector<double> eK, eS, Xn((size_t)nen * 3), meenDummy;
  std::vector<int> meen;
  Basis1D b[3];
  for (int iel = 0; iel < pc.nelAll; iel++) {
    if (pc.mnpc[iel].empty()) continue;
    const int ee[3] = {iel % pc.nel_d[0], (iel / pc.nel_d[0]) % pc.nel_d[1],
                       iel / (pc.nel_d[0] * pc.nel_d[1])};
    if (faceDir < 0 && ee[nd0] != 0) continue;
    if (faceDir > 0 && ee[nd0] != pc.nel_d[nd0] - 1) continue;
    const auto& nodes = pc.mnpc[iel];
    double dA = 0.25;
    for (int d = 0; d < 3; d++)
      if (d != nd0) dA *= pc.U[d][pc.p[d] + ee[d] + 1] - pc.U[d][pc.p[d] + ee[d]];
    for (int a = 0; a < nen; a++)
      for (int c = 0; c < 3; c++) Xn[(size_t)a * 3 + c] = pc.X[(size_t)nodes[a] * 3 + c];
    eS.assign((size_t)nen * npv, 0.0);
    for (int k = 0; k < ng[2]; k++)
      for (int j = 0; j < ng[1]; j++)
        for (int i = 0; i < ng[0]; i++) {
          const int gi[3] = {i, j, k};
          double wt = dA;
          for (int d = 0; d < 3; d++) {
            double u;
            if (d == nd0)
              u = faceDir < 0 ? pc.U[d][pc.p[d]] : pc.U[d][pc.n[d]];
            else {
              u = gaussParam(pc, d, ee[d], xg[d][gi[d]]);
              wt *= wg[d][gi[d]];
            }
            eval1D(pc, d, pc.p[d] + ee[d], u, b[d]);
          }
          tensorBasis(pc, b, nodes, s.N, s.dNdu);
          double normal[3];
          double dS = faceJacobian(nen, Xn.data(), s.dNdu.data(), t1, t2, normal);
          if (dS == 0.0) continue;
          double detJxW = dS * wt;
          for (int a = 0; a < nen; a++)
            for (int c = 0; c < npv; c++) eS[(size_t)a * npv + c] += nm.t[c] * s.N[a] * detJxW;
        }
    // SAM::assembleSystem(b, eS, iel): free DOFs only
    getElmEqns(m, pc.mlge[iel], meen);
    for (size_t i = 0; i < meen.size(); i++)
      if (meen[i] > 0) m.b[meen[i] - 1] += eS[i];
  }
}

// Two stripe groups along the direction with most elements, one stripe per
// thread and group (ThreadGroups::calcGroups, src/Utility/ThreadGroups.C:88-181,
// :253-...), so that threads of one group never share nodes.
void threadGroups(const Patch& pc, int threads, std::vector<std::vector<std::vector<int>>>& g)
{
  g.clear();
  int dir = 0;
  for (int d = 1; d < pc.dim; d++)
    if (pc.nel_d[d] > pc.nel_d[dir]) dir = d;
  const int els = pc.nel_d[dir], minsize = pc.p[dir];
  int parts = 2 * threads, stripsize = 0;
  while (threads > 1 && (stripsize = els / parts) < minsize) { threads--; parts -= 2; }
  if (threads <= 1) {
    g.assign(1, std::vector<std::vector<int>>(1));
    for (int e = 0; e < pc.nelAll; e++) g[0][0].push_back(e);
    return;
  }
  std::vector<int> sizes(parts, stripsize);
  int rem = els - stripsize * parts;
  for (int i = 0; i < rem; i++) sizes[parts - 1 - i]++;
  g.assign(2, std::vector<std::vector<int>>(threads));
  int start = 0;
  for (int s = 0; s < parts; s++) {
    auto& lst = g[s % 2][s / 2];
    for (int e = 0; e < pc.nelAll; e++) {
      int idx[3] = {e % pc.nel_d[0], (e / pc.nel_d[0]) % pc.nel_d[1],
                    e / (pc.nel_d[0] * pc.nel_d[1])};
      if (idx[dir] >= start && idx[dir] < start + sizes[s]) lst.push_back(e);
    }
    start += sizes[s];
  }
}

}  // namespace

// ===========================================================================
// C API used by the tests and the CPU baseline (ctypes).
// ===========================================================================
extern "C" {

void* ifo_create(int nGauss)
{
  Model* m = new Model;
  m->nGauss = nGauss;
  return m;
}

void ifo_destroy(void* h) { delete static_cast<Model*>(h); }

void ifo_set_bisect(void* h, int on) { static_cast<Model*>(h)->bisect = on != 0; }

int ifo_add_patch(void* h, int dim, const int* degree, const int* ncoef,
                  const double* const* knots, const double* coefs, int rational)
{
  Model& m = *static_cast<Model*>(h);
  Patch pc;
  pc.dim = dim;
  int nn = 1;
  for (int d = 0; d < dim; d++) {
    pc.p[d] = degree[d];
    pc.n[d] = ncoef[d];
    pc.U[d].assign(knots[d], knots[d] + ncoef[d] + degree[d] + 1);
    nn *= ncoef[d];
  }
  const int stride = dim + (rational ? 1 : 0);
  pc.X.resize((size_t)nn * dim);
  pc.W.assign(nn, 1.0);
  pc.rational = rational != 0;
  for (int i = 0; i < nn; i++) {
    for (int c = 0; c < dim; c++) pc.X[(size_t)i * dim + c] = coefs[(size_t)i * stride + c];
    if (rational) pc.W[i] = coefs[(size_t)i * stride + dim];
  }
  m.patches.push_back(pc);
  return (int)m.patches.size();
}

int ifo_set_material(void* h, int pid, int kind, double kappa, double source,
                     int source_shape, double E, double nu, const double* body)
{
  Model& m = *static_cast<Model*>(h);
  Patch& pc = m.patches.at(pid - 1);
  pc.mat.kind = kind;
  pc.mat.kappa = kappa;
  pc.mat.source = source;
  pc.mat.source_shape = source_shape;
  pc.mat.E = E;
  pc.mat.nu = nu;
  for (int c = 0; c < 3; c++) pc.mat.body[c] = body ? body[c] : 0.0;
  pc.npv = kind == 2 ? pc.dim : 1;
  return 0;
}

int ifo_connect(void* h, int master, int mface, int slave, int sface, int orient)
{
  static_cast<Model*>(h)->conns.push_back({master, mface, slave, sface, orient});
  return 0;
}

int ifo_set_mass(void* h, int pid, double scale)
{
  static_cast<Model*>(h)->patches.at(pid - 1).mat.mass = scale;
  return 0;
}

int ifo_set_field(void* h, int pid, int which, const double* v)
{
  Model& m = *static_cast<Model*>(h);
  Patch& pc = m.patches.at(pid - 1);
  int nn = (int)pc.W.size();
  if (which == 1) pc.logk.assign(v, v + nn); else pc.noise.assign(v, v + nn);
  return 0;
}

int ifo_constrain_face(void* h, int pid, int face, int dofs, double value)
{
  Model& m = *static_cast<Model*>(h);
  m.patches.at(pid - 1).bcs.push_back({face, dofs, value});
  return 0;
}

int ifo_add_neumann(void* h, int pid, int face, const double* t)
{
  Model& m = *static_cast<Model*>(h);
  Neumann nm{face, {0, 0, 0}};
  Patch& pc = m.patches.at(pid - 1);
  for (int c = 0; c < pc.npv; c++) nm.t[c] = t[c];
  pc.neumann.push_back(nm);
  return 0;
}

// mode 0: IFEM's std::set couplings (buildPattern), mode 1: the parallel
// node-neighbour construction (buildPatternFast), -1: the latter for models
// with more than 5e7 element-matrix entries.  Both give the same arrays.
int ifo_preprocess(void* h, int mode)
{
  Model& m = *static_cast<Model*>(h);
  if (!initSAM(m)) return -1;
  long long work = 0;
  for (int iel = 1; iel <= m.nel; iel++) {
    long long nd = 0;
    for (int ip = m.mpmnpc[iel - 1]; ip < m.mpmnpc[iel]; ip++) {
      const int node = m.mmnpc[ip - 1];
      nd += m.madof[node] - m.madof[node - 1];
    }
    work += nd * nd;
  }
  if (mode == 1 || (mode < 0 && work > 50000000LL))
    buildPatternFast(m);
  else
    buildPattern(m);
  return 0;
}

void ifo_sizes(void* h, int* out)
{
  Model& m = *static_cast<Model*>(h);
  out[0] = m.nnod; out[1] = m.nel; out[2] = m.ndof; out[3] = m.neq; out[4] = m.nceq;
  out[5] = (int)m.JA.size();
}

void ifo_get_sam(void* h, int* madof, int* meqn)
{
  Model& m = *static_cast<Model*>(h);
  std::memcpy(madof, m.madof.data(), sizeof(int) * m.madof.size());
  std::memcpy(meqn, m.meqn.data(), sizeof(int) * m.meqn.size());
}

void ifo_get_pattern(void* h, int* IA, int* JA)
{
  Model& m = *static_cast<Model*>(h);
  std::memcpy(IA, m.IA.data(), sizeof(int) * m.IA.size());
  std::memcpy(JA, m.JA.data(), sizeof(int) * m.JA.size());
}

int ifo_get_mnpc(void* h, int pid, int* out)
{
  Model& m = *static_cast<Model*>(h);
  Patch& pc = m.patches.at(pid - 1);
  int nen = pc.nen(), k = 0;
  for (int e = 0; e < pc.nelAll; e++)
    for (int a = 0; a < nen; a++)
      out[k++] = pc.mnpc[e].empty() ? -1 : pc.mnpc[e][a];
  return pc.nelAll;
}

// Assembly of all patches.  threads <= 1: element order of a serial IFEM
// build (parity mode).  threads > 1: OpenMP over the stripe groups as the
// reference does with USE_OPENMP (baseline mode).  Returns the number of
// skipped singular integration points; max_elements > 0 limits the number of
// elements per patch (bounded baseline sample).
long ifo_assemble(void* h, int threads, long max_elements)
{
  Model& m = *static_cast<Model*>(h);
  // SystemMatrix::init / SystemVector::init (zeroing), on every thread
  const long long nA = (long long)m.A.size();
#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : 1)
  for (long long i = 0; i < nA; i++) m.A[i] = 0.0;
  std::fill(m.b.begin(), m.b.end(), 0.0);
  long singular = 0;
  for (auto& pc : m.patches) {
    int ng[3] = {1, 1, 1};
    std::vector<double> xgv[3], wgv[3];
    const double* xg[3] = {nullptr, nullptr, nullptr};
    const double* wg[3] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < pc.dim; d++) {
      ng[d] = numGauss(m, pc.p[d] + 1, false);
      xgv[d].resize(ng[d]);
      wgv[d].resize(ng[d]);
      gaussLegendre(ng[d], xgv[d].data(), wgv[d].data());
      xg[d] = xgv[d].data();
      wg[d] = wgv[d].data();
    }
    long limit = max_elements > 0 ? std::min<long>(max_elements, pc.nelAll) : pc.nelAll;
    if (threads <= 1) {
      Scratch s;
      std::vector<double> eK, eS;
      std::vector<int> meen;
      for (long e = 0; e < limit; e++)
        singular += integrateElement(m, pc, (int)e, ng, xg, wg, s, eK, eS, meen, true);
    } else {
#ifdef _OPENMP
      std::vector<std::vector<std::vector<int>>> groups;
      threadGroups(pc, threads, groups);
      for (auto& grp : groups) {
#pragma omp parallel for schedule(static) num_threads(threads) reduction(+:singular)
        for (int t = 0; t < (int)grp.size(); t++) {
          Scratch s;
          std::vector<double> eK, eS;
          std::vector<int> meen;
          for (int e : grp[t])
            if (e < limit)
              singular += integrateElement(m, pc, e, ng, xg, wg, s, eK, eS, meen, true);
        }
      }
#endif
    }
    for (auto& nm : pc.neumann) integrateNeumann(m, pc, nm);
  }
  return singular;
}

// Element matrices only (no scatter): eK (nd x nd, column-major) and eS of
// element iel (0-based, patch-local).  Returns nd, or -1 for an empty element.
int ifo_element(void* h, int pid, int iel, double* eKout, double* eSout)
{
  Model& m = *static_cast<Model*>(h);
  Patch& pc = m.patches.at(pid - 1);
  if (pc.mnpc[iel].empty()) return -1;
  int ng[3] = {1, 1, 1};
  std::vector<double> xgv[3], wgv[3];
  const double* xg[3] = {nullptr, nullptr, nullptr};
  const double* wg[3] = {nullptr, nullptr, nullptr};
  for (int d = 0; d < pc.dim; d++) {
    ng[d] = numGauss(m, pc.p[d] + 1, false);
    xgv[d].resize(ng[d]); wgv[d].resize(ng[d]);
    gaussLegendre(ng[d], xgv[d].data(), wgv[d].data());
    xg[d] = xgv[d].data(); wg[d] = wgv[d].data();
  }
  Scratch s;
  std::vector<double> eK, eS;
  std::vector<int> meen;
  integrateElement(m, pc, iel, ng, xg, wg, s, eK, eS, meen, false);
  std::memcpy(eKout, eK.data(), sizeof(double) * eK.size());
  std::memcpy(eSout, eS.data(), sizeof(double) * eS.size());
  return (int)eS.size();
}

// Norm totals and per-element norms (patches in order, all elements of a
// patch first index fastest); the secondary solution of one patch.
void ifo_norms(void* h, const double* u, double* totals, double* elem)
{
  Model& m = *static_cast<Model*>(h);
  totals[0] = totals[1] = 0.0;
  size_t slot = 0;
  for (Patch& pc : m.patches)
    for (int e = 0; e < pc.nelAll; e++, slot++) {
      double o[2];
      elementNorms(m, pc, e, u, o, nullptr);
      totals[0] += o[0];
      totals[1] += o[1];
      if (elem) {
        elem[2 * slot] = o[0];
        elem[2 * slot + 1] = o[1];
      }
    }
}

void ifo_secondary(void* h, int pid, const double* u, double* out)
{
  Model& m = *static_cast<Model*>(h);
  Patch& pc = m.patches.at(pid - 1);
  int nq = 1;
  for (int d = 0; d < pc.dim; d++) nq *= numGauss(m, pc.p[d] + 1, false);
  const int nc = pc.mat.kind == 1 ? pc.dim : 6;
  for (int e = 0; e < pc.nelAll; e++) {
    double o[2];
    elementNorms(m, pc, e, u, o, out + (size_t)e * nq * nc);
  }
}

void ifo_get_system(void* h, double* A, double* b)
{
  Model& m = *static_cast<Model*>(h);
  std::memcpy(A, m.A.data(), sizeof(double) * m.A.size());
  std::memcpy(b, m.b.data(), sizeof(double) * m.b.size());
}

// ---- element-level kernels exposed for the golden tests -------------------

void ifo_gauss(int n, double* xi, double* w) { gaussLegendre(n, xi, w); }

// Basis values N (nen) and dNdu (nen x dim col-major) of a patch at a
// parameter point, evaluated on the span that contains it (GoTools rule).
int ifo_basis(void* h, int pid, const double* u, double* N, double* dNdu, int* nodesOut)
{
  Model& m = *static_cast<Model*>(h);
  Patch& pc = m.patches.at(pid - 1);
  Basis1D b[3];
  int span[3] = {0, 0, 0};
  for (int d = 0; d < pc.dim; d++) {
    span[d] = findSpan(pc.n[d], pc.p[d], u[d], pc.U[d].data());
    eval1D(pc, d, span[d], u[d], b[d]);
  }
  std::vector<int> nodes;
  const int q1 = pc.p[0] + 1, q2 = pc.p[1] + 1, q3 = pc.dim == 3 ? pc.p[2] + 1 : 1;
  for (int k = 0; k < q3; k++)
    for (int j = 0; j < q2; j++)
      for (int i = 0; i < q1; i++) {
        int I = span[0] - pc.p[0] + i, J = span[1] - pc.p[1] + j;
        int K = pc.dim == 3 ? span[2] - pc.p[2] + k : 0;
        nodes.push_back((K * pc.n[1] + J) * pc.n[0] + I);
      }
  std::vector<double> Nv, dN;
  tensorBasis(pc, b, nodes, Nv, dN);
  std::memcpy(N, Nv.data(), sizeof(double) * Nv.size());
  std::memcpy(dNdu, dN.data(), sizeof(double) * dN.size());
  if (nodesOut) std::memcpy(nodesOut, nodes.data(), sizeof(int) * nodes.size());
  return (int)nodes.size();
}

double ifo_jacobian(int dim, int nen, const double* Xn, const double* dNdu,
                    double* J, double* dNdX)
{
  return jacobian(dim, nen, Xn, dNdu, J, dNdX);
}

// Element operators on given dNdX (nen x dim col-major) and N, detJxW.
void ifo_op_laplacian(int dim, int nen, const double* dNdX, double kappa,
                      double detJxW, double* eK)
{
  for (int j = 0; j < nen; j++)
    for (int i = 0; i < nen; i++) {
      double v = 0.0;
      for (int c = 0; c < dim; c++)
        v += dNdX[(size_t)c * nen + i] * kappa * detJxW * dNdX[(size_t)c * nen + j];
      eK[(size_t)j * nen + i] += v;
    }
}

// Isotropic elasticity operator for dim=2 (plane strain) or 3, written in the
// component form lam*div.div + mu*(grad:grad + grad^T:grad).
void ifo_op_elasticity(int dim, int nen, const double* dNdX, double lam, double mu,
                       double detJxW, double* eK)
{
  const int nd = dim * nen;
  for (int a = 0; a < nen; a++)
    for (int b = 0; b < nen; b++)
      for (int k = 0; k < dim; k++)
        for (int l = 0; l < dim; l++) {
          double g = 0.0;
          for (int c = 0; c < dim; c++) g += dNdX[(size_t)c * nen + a] * dNdX[(size_t)c * nen + b];
          double v = lam * dNdX[(size_t)k * nen + a] * dNdX[(size_t)l * nen + b] +
                     mu * dNdX[(size_t)l * nen + a] * dNdX[(size_t)k * nen + b] +
                     (k == l ? mu * g : 0.0);
          eK[(size_t)(dim * b + l) * nd + dim * a + k] += v * detJxW;
        }
}

// ---- FP64 Jacobi-PCG on the assembled compressed-column system -----------
// (symmetric: CSC == CSR).  Used as the CPU solve baseline for systems where
// a direct solve is out of reach.  Returns iterations, relres in *relres.
int ifo_pcg(void* h, const double* b, double* x, double rtol, int maxit,
            int threads, double* relres)
{
  Model& m = *static_cast<Model*>(h);
  const int n = m.neq;
  const int nt = threads > 0 ? threads : 1;
  std::vector<double> r(n), z(n), p(n), q(n), dinv(n);
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int j = 0; j < n; j++) {
    dinv[j] = 1.0;
    for (int k = m.IA[j]; k < m.IA[j + 1]; k++)
      if (m.JA[k] == j) dinv[j] = 1.0 / m.A[k];
  }
  auto spmv = [&](const std::vector<double>& v, std::vector<double>& out) {
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int j = 0; j < n; j++) {
      double s = 0.0;
      for (int k = m.IA[j]; k < m.IA[j + 1]; k++) s += m.A[k] * v[m.JA[k]];
      out[j] = s;
    }
  };
  std::vector<double> xv(x, x + n);
  spmv(xv, q);
  double bn = 0.0, rz = 0.0;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(+:bn, rz)
  for (int i = 0; i < n; i++) {
    r[i] = b[i] - q[i];
    bn += b[i] * b[i];
    z[i] = dinv[i] * r[i];
    p[i] = z[i];
    rz += r[i] * z[i];
  }
  bn = std::sqrt(bn);
  if (bn == 0.0) bn = 1.0;
  int it = 0;
  double rn = 0.0;
  for (; it < maxit; it++) {
    rn = 0.0;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(+:rn)
    for (int i = 0; i < n; i++) rn += r[i] * r[i];
    if (std::sqrt(rn) / bn <= rtol) break;
    spmv(p, q);
    double pq = 0.0;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(+:pq)
    for (int i = 0; i < n; i++) pq += p[i] * q[i];
    double alpha = rz / pq, rz1 = 0.0;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(+:rz1)
    for (int i = 0; i < n; i++) {
      xv[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      z[i] = dinv[i] * r[i];
      rz1 += r[i] * z[i];
    }
    double beta = rz1 / rz;
    rz = rz1;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
  }
  // true residual
  spmv(xv, q);
  rn = 0.0;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(+:rn)
  for (int i = 0; i < n; i++) rn += (b[i] - q[i]) * (b[i] - q[i]);
  *relres = std::sqrt(rn) / bn;
  std::memcpy(x, xv.data(), sizeof(double) * n);
  return it;
}

}  // extern "C"
