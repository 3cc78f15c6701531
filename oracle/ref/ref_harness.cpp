// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Drives IFEM's own numbering, sparsity, Jacobian, weak-form and assembly code
// (compiled unmodified from the IFEM sources by oracle/ref/build_ref.py) on a
// structured patch whose topology and basis values come from the outside:
//
//   * GridPatch: an ASMbase with given MNPC, the part of ASMs3D/ASMs2D
//     (src/ASM/ASMs3D.C:433-516, :3899-3924) that needs GoTools replaced by
//     plain arrays; Dirichlet DOFs via ASMbase::fix (src/ASM/ASMbase.C:963);
//   * SAMpatch::init (src/ASM/SAMpatch.C:21-81) -> MADOF, MEQN;
//   * SparseMatrix(SUPERLU)::initAssembly(sam, 'F') (src/LinAlg/SparseMatrix.C:
//     717-762) -> the locked compressed-column pattern of optimiseCols;
//   * per Gauss point utl::Jacobian (src/Utility/CoordinateMapping.C:24-63),
//     EqualOrderOperators::Weak::Laplacian / Mass / Source (Apps/Utils/
//     EqualOrderOperators.C:158-174, :214-227, :243-254) -- the loop body of
//     ASMs3D::integrate (src/ASM/ASMs3D.C:2266-2312) restated here;
//   * SAM::assembleSystem (src/LinAlg/SAM.C:430-543) into the SparseMatrix
//     and a StdVector.
//
// Basis values (IFEM obtains them from GoTools, absent here) are inputs.
// The library built from this file is the checker of the CPU oracle; nothing
// of the product links it.
#include <cstring>
#include <fstream>
#include <iomanip>
#include <map>
#include <vector>

#include "ASMbase.h"
#include "CoordinateMapping.h"
#include "EqualOrderOperators.h"
#include "FiniteElement.h"
#include "GaussQuadrature.h"
#include "LinAlgenums.h"
#include "MatVec.h"
#include "SAMpatch.h"
#include "SparseMatrix.h"
#include "SystemMatrix.h"
#include "Vec3.h"

#define RH_API extern "C" __attribute__((visibility("default")))

namespace {

class GridPatch : public ASMbase
{
public:
  GridPatch(int dim, int nfield, int nnodes, int nelem, int nen, const int* mnpc)
    : ASMbase(dim, dim, nfield)
  {
    nnod = nnodes;
    nel = nelem;
    myMLGN.resize(nnodes);
    for (int i = 0; i < nnodes; i++) myMLGN[i] = i + 1;
    myMLGE.resize(nelem);
    for (int e = 0; e < nelem; e++) myMLGE[e] = e + 1;
    myMNPC.assign(nelem, IntVec(nen));
    for (int e = 0; e < nelem; e++)
      for (int a = 0; a < nen; a++) myMNPC[e][a] = mnpc[(size_t)e * nen + a];
  }

  int fixNode(size_t inod, int dirs) { return this->fix(inod, dirs); }
  void setGlobal(int firstNode, int firstElm)
  {
    for (size_t i = 0; i < myMLGN.size(); i++) myMLGN[i] = firstNode + (int)i + 1;
    for (size_t e = 0; e < myMLGE.size(); e++) myMLGE[e] = firstElm + (int)e + 1;
  }
  // ASMbase::collapseNodes and addNeighbor, as ASMs3D::connectBasis /
  // connectPatch use them (protected in ASMbase)
  static bool collapse(GridPatch& master, int mnode, GridPatch& slave, int snode)
  {
    return ASMbase::collapseNodes(master, mnode, slave, snode);
  }
  void neighbour(GridPatch* other) { this->addNeighbor(other); }

  bool empty() const override { return false; }
  bool read(std::istream&) override { return false; }
  bool write(std::ostream&, int) const override { return false; }
  bool generateFEMTopology() override { return true; }
  Vec3 getCoord(size_t) const override { return Vec3(); }
  void getNodalCoordinates(Matrix&, bool) const override {}
  Vec3 getElementCenter(int) const override { return Vec3(); }
  bool updateCoords(const Vector&) override { return false; }
  bool integrate(Integrand&, GlobalIntegral&, const TimeDomain&) override { return false; }
  bool integrate(Integrand&, int, GlobalIntegral&, const TimeDomain&) override { return false; }
  int evalPoint(const double*, double*, Vec3&) const override { return -1; }
  int findElementContaining(const double*) const override { return -1; }
  double findPoint(Vec3&, double*) const override { return -1.0; }
  bool tesselate(ElementBlock&, const int*) const override { return false; }
  void findBoundaryElms(IntVec&, int, int) const override {}
  bool getElementCoordinates(Matrix&, int, bool) const override { return false; }
  void getBoundaryNodes(int, IntVec&, int, int, int, bool) const override {}
  bool getParameterDomain(Real2DMat&, IntVec*) const override { return false; }
  void getElmConnectivities(IntMat&, int) const override {}
};

// read access to the compressed-column arrays (protected in SparseMatrix)
class CscView : public SparseMatrix
{
public:
  using SparseMatrix::SparseMatrix;
  const IntVec& colPtr() const { return IA; }
  const IntVec& rowIdx() const { return JA; }
  const std::vector<Real>& values() const { return A; }
};

struct Harness
{
  GridPatch* patch = nullptr;        // first patch (single-patch models)
  std::vector<GridPatch*> patches;   // all patches, owned
  std::vector<int> firstElm;         // global element offset per patch
  int nnodGlobal = 0;
  SAMpatch sam;
  CscView K{SparseMatrix::SUPERLU};
  StdVector b;
  int dim = 3, nf = 1, nen = 0;
  ~Harness()
  {
    if (patches.empty()) delete patch;
    for (GridPatch* p : patches) delete p;
  }
};

}  // namespace

// MNPC: nel x nen 0-based patch node indices (IFEM's local order)
RH_API void* rh_create(int dim, int nf, int nnod, int nel, int nen, const int* mnpc)
{
  Harness* h = new Harness;
  h->dim = dim;
  h->nf = nf;
  h->nen = nen;
  h->patch = new GridPatch(dim, nf, nnod, nel, nen, mnpc);
  return h;
}

RH_API void rh_destroy(void* p) { delete static_cast<Harness*>(p); }

// homogeneous Dirichlet code (e.g. 123) on 1-based node inod; returns the
// ignored directions as ASMbase::fix does
RH_API int rh_fix(void* p, int inod, int dirs)
{
  return static_cast<Harness*>(p)->patch->fixNode(inod, dirs);
}

// Multi-patch model: npatch patches with nnod[i] nodes, nel[i] elements of
// nen nodes each and MNPC (0-based patch nodes, patches one after the
// other); global node and element numbers start consecutive per patch, as
// ASMs3D::generateFEMTopology assigns them.
RH_API void* rh_create_multi(int dim, int nf, int npatch, const int* nnod, const int* nel, int nen,
                             const int* mnpc)
{
  Harness* h = new Harness;
  h->dim = dim;
  h->nf = nf;
  h->nen = nen;
  int gn = 0, ge = 0;
  for (int i = 0; i < npatch; i++) {
    GridPatch* g = new GridPatch(dim, nf, nnod[i], nel[i], nen, mnpc);
    g->setGlobal(gn, ge);
    h->firstElm.push_back(ge);
    gn += nnod[i];
    ge += nel[i];
    mnpc += (size_t)nel[i] * nen;
    h->patches.push_back(g);
  }
  h->patch = h->patches.front();
  h->nnodGlobal = gn;
  return h;
}

// One node pair of a connection (1-based patch-local nodes), then, after the
// last pair of a connection, the neighbour registration of connectPatch.
RH_API int rh_collapse(void* p, int master, int mnode, int slave, int snode)
{
  Harness* h = static_cast<Harness*>(p);
  return GridPatch::collapse(*h->patches[master - 1], mnode, *h->patches[slave - 1], snode);
}

RH_API void rh_neighbours(void* p, int master, int slave)
{
  Harness* h = static_cast<Harness*>(p);
  h->patches[slave - 1]->neighbour(h->patches[master - 1]);
}

// SIMbase::renumberNodes (src/SIM/SIMbase.C:535-565) with preserveNOrder
// off: numbers compacted patch by patch in order of first appearance.
RH_API int rh_renumber(void* p)
{
  Harness* h = static_cast<Harness*>(p);
  std::map<int, int> old2new;
  int nnod = 0;
  for (GridPatch* g : h->patches) g->renumberNodes(old2new, nnod);
  h->nnodGlobal = nnod;
  return nnod;
}

// homogeneous Dirichlet code on 1-based patch-local node inod of patch pid
RH_API int rh_fix_patch(void* p, int pid, int inod, int dirs)
{
  return static_cast<Harness*>(p)->patches[pid - 1]->fixNode(inod, dirs);
}

// the global node number (1-based) of patch-local node inod (1-based)
RH_API int rh_node_id(void* p, int pid, int inod)
{
  return static_cast<Harness*>(p)->patches[pid - 1]->getNodeID(inod);
}

// global element number (1-based) of patch-local element iel (0-based)
RH_API int rh_elm_id(void* p, int pid, int iel)
{
  return static_cast<Harness*>(p)->firstElm[pid - 1] + iel + 1;
}

// SAM numbering and the locked pattern; out = {nnod, ndof, neq, nnz}
RH_API int rh_init(void* p, int* out)
{
  Harness* h = static_cast<Harness*>(p);
  std::vector<ASMbase*> model;
  if (h->patches.empty()) model.push_back(h->patch);
  for (GridPatch* g : h->patches) model.push_back(g);
  if (!h->sam.init(model, h->patches.empty() ? 0 : h->nnodGlobal, {})) return -1;
  h->K.initAssembly(h->sam, 'F');
  h->b.redim(h->sam.getNoEquations());
  out[0] = h->sam.getNoNodes();
  out[1] = h->sam.getNoDOFs();
  out[2] = h->sam.getNoEquations();
  out[3] = (int)h->K.size();
  return 0;
}

RH_API void rh_gauss(int n, double* xi, double* w)
{
  const double* x = GaussQuadrature::getCoord(n);
  const double* g = GaussQuadrature::getWeight(n);
  for (int i = 0; i < n; i++) {
    xi[i] = x ? x[i] : 0.0;
    w[i] = g ? g[i] : 0.0;
  }
}

// One Poisson element (1-based iel) from its nq Gauss points: N[q][a],
// dNdu[q][d][a], wfac[q] = dV * w_i w_j (w_k), kappa[q], f[q]; the scale of
// the mass matrix added to K (0: none) and the element's control points
// X[a][3].  Forms eK, eS with IFEM's operators, assembles them and returns
// them (eK column-major); the return value is the number of points skipped
// for a singular Jacobian.
RH_API int rh_poisson_element(void* p, int iel, int nq, const double* N, const double* dNdu,
                              const double* wfac, const double* kappa, const double* f,
                              double mass, const double* X, double* eKout, double* eSout)
{
  Harness* h = static_cast<Harness*>(p);
  const int nen = h->nen, dim = h->dim;
  Matrix Xnod(dim, nen);  // nsd = dim for these patches
  for (int a = 0; a < nen; a++)
    for (int r = 0; r < dim; r++) Xnod(r + 1, a + 1) = X[(size_t)a * 3 + r];
  Matrix eK(nen, nen);
  Vector eS(nen);
  FiniteElement fe(nen);
  Matrix J, dNdu_m(nen, dim);
  int skipped = 0;
  for (int q = 0; q < nq; q++) {
    for (int a = 0; a < nen; a++) {
      fe.N(a + 1) = N[(size_t)q * nen + a];
      for (int d = 0; d < dim; d++) dNdu_m(a + 1, d + 1) = dNdu[((size_t)q * dim + d) * nen + a];
    }
    const double detJ = utl::Jacobian(J, fe.dNdX, Xnod, dNdu_m);
    if (detJ == 0.0) {
      skipped++;
      continue;
    }
    fe.detJxW = detJ * wfac[q];
    EqualOrderOperators::Weak::Laplacian(eK, fe, kappa[q]);
    if (mass != 0.0) EqualOrderOperators::Weak::Mass(eK, fe, mass);
    EqualOrderOperators::Weak::Source(eS, fe, f[q]);
  }
  h->sam.assembleSystem(h->K, h->b, eK, iel);
  h->sam.assembleSystem(h->b, eS, iel);
  for (int j = 0; j < nen; j++)
    for (int i = 0; i < nen; i++) eKout[(size_t)j * nen + i] = eK(i + 1, j + 1);
  for (int i = 0; i < nen; i++) eSout[i] = eS(i + 1);
  return skipped;
}

// Secondary solution at the Gauss points of one element from IFEM's
// utl::Jacobian (src/Utility/CoordinateMapping.C:24-63): per point q the
// spatial gradients dNdX of the element functions, then for Poisson (nf = 1)
// the flux -kappa[q] grad u, for isotropic elasticity (nf = dim = 3) the
// stress lambda tr(eps) I + 2 mu eps in Voigt order xx yy zz xy yz zx, from
// the element's solution values ue[a][c].  N[q][a], dNdu[q][d][a], X[a][3] as
// for rh_poisson_element; out[q][.]; zero at singular points.  The
// application integrands that evaluate these (IFEM-Poisson, IFEM-Elasticity)
// are outside the IFEM tree; the constitutive step is the same one the
// element matrices use.
RH_API int rh_secondary_points(int dim, int nen, int nq, const double* N, const double* dNdu,
                               const double* X, int nf, const double* ue, const double* kappa,
                               double lam, double mu, double* out)
{
  Matrix Xnod(dim, nen);
  for (int a = 0; a < nen; a++)
    for (int r = 0; r < dim; r++) Xnod(r + 1, a + 1) = X[(size_t)a * 3 + r];
  Matrix J, dNdX, dNdu_m(nen, dim);
  const int ncomp = nf == 1 ? dim : 6;
  int skipped = 0;
  for (int q = 0; q < nq; q++) {
    (void)N;
    for (int a = 0; a < nen; a++)
      for (int d = 0; d < dim; d++) dNdu_m(a + 1, d + 1) = dNdu[((size_t)q * dim + d) * nen + a];
    double* o = out + (size_t)q * ncomp;
    for (int c = 0; c < ncomp; c++) o[c] = 0.0;
    const double detJ = utl::Jacobian(J, dNdX, Xnod, dNdu_m);
    if (detJ == 0.0) {
      skipped++;
      continue;
    }
    if (nf == 1) {
      for (int k = 0; k < dim; k++) {
        double g = 0.0;
        for (int a = 0; a < nen; a++) g += dNdX(a + 1, k + 1) * ue[a];
        o[k] = -kappa[q] * g;
      }
    } else {
      double G[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // G[c][k] = du_c/dx_k
      for (int a = 0; a < nen; a++)
        for (int c = 0; c < 3; c++)
          for (int k = 0; k < 3; k++) G[c][k] += ue[(size_t)a * 3 + c] * dNdX(a + 1, k + 1);
      const double tr = G[0][0] + G[1][1] + G[2][2];
      o[0] = lam * tr + 2.0 * mu * G[0][0];
      o[1] = lam * tr + 2.0 * mu * G[1][1];
      o[2] = lam * tr + 2.0 * mu * G[2][2];
      o[3] = mu * (G[0][1] + G[1][0]);
      o[4] = mu * (G[1][2] + G[2][1]);
      o[5] = mu * (G[2][0] + G[0][2]);
    }
  }
  return skipped;
}

// Assemble a given element matrix (column-major, nd x nd with nd = nf * nen)
// and load vector through SAM::assembleSystem.
RH_API int rh_assemble(void* p, int iel, const double* eKin, const double* eSin)
{
  Harness* h = static_cast<Harness*>(p);
  const int nd = h->nf * h->nen;
  Matrix eK(nd, nd);
  Vector eS(nd);
  for (int j = 0; j < nd; j++)
    for (int i = 0; i < nd; i++) eK(i + 1, j + 1) = eKin[(size_t)j * nd + i];
  for (int i = 0; i < nd; i++) eS(i + 1) = eSin[i];
  bool ok = h->sam.assembleSystem(h->K, h->b, eK, iel);
  ok = ok && h->sam.assembleSystem(h->b, eS, iel);
  return ok ? 0 : -1;
}

RH_API void rh_get_sam(void* p, int* madof, int* meqn)
{
  Harness* h = static_cast<Harness*>(p);
  const int nnod = h->sam.getNoNodes(), ndof = h->sam.getNoDOFs();
  std::memcpy(madof, h->sam.getMADOF(), sizeof(int) * (nnod + 1));
  std::memcpy(meqn, h->sam.getMEQN(), sizeof(int) * ndof);
}

// IA (neq+1), JA (nnz) 0-based as SparseMatrix stores them, values, rhs
RH_API void rh_get_system(void* p, int* IA, int* JA, double* A, double* b)
{
  Harness* h = static_cast<Harness*>(p);
  const IntVec& ia = h->K.colPtr();
  const IntVec& ja = h->K.rowIdx();
  const std::vector<Real>& a = h->K.values();
  std::memcpy(IA, ia.data(), sizeof(int) * ia.size());
  std::memcpy(JA, ja.data(), sizeof(int) * ja.size());
  std::memcpy(A, a.data(), sizeof(double) * a.size());
  for (size_t i = 0; i < h->b.size(); i++) b[i] = h->b[i];
}

// The system written by IFEM's own SparseMatrix::dump / StdVector::dump the
// way SIMbase::dumpEqSys does (src/SIM/SIMbase.C:2863-2925): precision 17,
// labels "A" and "b", utl::zero_print_tol = zero_tol.
RH_API int rh_dump(void* p, const char* matrixPath, const char* rhsPath, int format,
                   double zeroTol)
{
  Harness* h = static_cast<Harness*>(p);
  const double old = utl::zero_print_tol;
  utl::zero_print_tol = zeroTol;
  if (matrixPath) {
    std::ofstream os(matrixPath);
    os << std::setprecision(17);
    h->K.dump(os, static_cast<LinAlg::StorageFormat>(format), "A");
  }
  if (rhsPath) {
    std::ofstream os(rhsPath);
    os << std::setprecision(17);
    h->b.dump(os, static_cast<LinAlg::StorageFormat>(format), "b");
  }
  utl::zero_print_tol = old;
  return 0;
}
