// GpuSIM3D.h -- the IFEM-side adapter of libifemgpu: a SIM3D whose assembly
// and linear solve run on the GPU through the C ABI in include/ifemgpu.h.
//
// It overrides the three virtuals of IFEM's simulator that the path sits
// behind, so that a SIM3D-based application (and IFEM's own drivers) picks
// the GPU up without changes to IFEM's sources:
//   SIMbase::preprocessB     (src/SIM/SIMbase.h:614)  the model goes to the
//                            GPU once IFEM's SAM is set up;
//   SIMbase::assembleSystem  (src/SIM/SIMbase.h:291)  replaces the patch
//                            loop over ASMs3D::integrate and SAM/assemSparse
//                            (src/SIM/SIMbase.C:1229-1429);
//   SIMbase::solveSystem     (src/SIM/SIMbase.h:334)  replaces solveEqSystem
//                            with SuperLU (src/SIM/SIMbase.C:1487-1550).
// IFEM's bool-and-stderr error convention is kept: a failing call prints
// " *** GpuSIM3D::<method>: <libifemgpu message>" and returns false.
//
// The spline data of a patch (degree, knot vectors and control net of its
// Go::SplineVolume) needs GoTools, so the adapter asks for it through the
// virtual splineData(), which an application implements with the GoTools
// accessors (Go::SplineVolume::order, basis(d).begin(), coefs_begin() /
// rcoefs_begin()).  Material constants and boundary conditions are set from
// the application's integrand and property sets through the setters below.
#ifndef IFEMGPU_ADAPTER_GPUSIM3D_H
#define IFEMGPU_ADAPTER_GPUSIM3D_H

#include <iostream>
#include <vector>

#include "ASMbase.h"
#include "SIM3D.h"
#include "TimeDomain.h"
#include "ifemgpu.h"

class GpuSIM3D : public SIM3D
{
public:
  //! \brief Spline description of one patch, first parametric index fastest.
  struct SplineData {
    int degree[3];                 //!< polynomial degree per direction
    int ncoef[3];                  //!< control points per direction
    std::vector<double> knots[3];  //!< ncoef + degree + 1 values per direction
    std::vector<double> coefs;     //!< x, y, z (and w when rational) per point
    bool rational = false;
  };

  //! \param[in] nf Number of unknowns per node (3: elasticity, 1: Poisson)
  //! \param[in] nGauss IFEM's nGauss (points per direction, or 10 + k)
  //! \param[in] split Split-precision element matrices on the tensor cores
  explicit GpuSIM3D(unsigned char nf = 3, int nGauss = 3, bool split = true) : SIM3D(nf)
  {
    ifemgpu_options o{0, split ? IFEMGPU_KE_SPLIT_TF32 : IFEMGPU_KE_FP64, nGauss, 0, 0};
    if (ifemgpu_ctx_create(&ctx, &o) != IFEMGPU_OK) ctx = nullptr;
    solver = ifemgpu_solver_options{IFEMGPU_PCG_MIXED, 1.0e-10, 20, 20000, 1.0e-4,
                                    IFEMGPU_PRECOND_KRONECKER};
  }
  ~GpuSIM3D() override { ifemgpu_ctx_destroy(ctx); }

  //! \brief Isotropic linear elasticity (or, with kind IFEMGPU_POISSON, the
  //! conductivity kappa and source f) of every patch.
  void setMaterial(const ifemgpu_material& m) { material = m; }
  //! \brief Homogeneous or prescribed Dirichlet condition on a patch face
  //! (IFEM face index 1..6, DOF digits such as 123), as SIM3D::addConstraint.
  void addFaceConstraint(int patch, int face, int dofs, double value = 0.0)
  {
    faceBCs.push_back({patch, face, dofs, value});
  }
  //! \brief Constant traction (elasticity) or normal flux (Poisson) on a face.
  void addFaceLoad(int patch, int face, double t0, double t1 = 0.0, double t2 = 0.0)
  {
    faceLoads.push_back({patch, face, {t0, t1, t2}});
  }
  //! \brief Method, preconditioner and tolerances of solveSystem.
  void setSolver(const ifemgpu_solver_options& o) { solver = o; }

  //! \brief The spline of patch \a pch (1-based); GoTools accessors.
  virtual bool splineData(const ASMbase* pch, int patch, SplineData& out) const = 0;

  bool preprocessB() override
  {
    if (!ctx) return fail("preprocessB", "no GPU context");
    int idx = 0;
    for (const ASMbase* pch : this->getFEModel()) {
      SplineData s;
      if (!this->splineData(pch, ++idx, s)) return fail("preprocessB", "no spline data");
      const double* kn[3] = {s.knots[0].data(), s.knots[1].data(), s.knots[2].data()};
      int id = 0;
      if (ifemgpu_patch_add(ctx, 3, s.degree, s.ncoef, kn, s.coefs.data(), s.rational ? 1 : 0,
                            &id) != IFEMGPU_OK ||
          ifemgpu_patch_set_material(ctx, id, &material) != IFEMGPU_OK)
        return fail("preprocessB");
    }
    for (const FaceBC& c : faceBCs)
      if (ifemgpu_patch_constrain_face(ctx, c.patch, c.face, c.dofs, c.value) != IFEMGPU_OK)
        return fail("preprocessB");
    for (const FaceLoad& l : faceLoads)
      if (ifemgpu_patch_add_neumann(ctx, l.patch, l.face, l.t) != IFEMGPU_OK)
        return fail("preprocessB");
    return ifemgpu_preprocess(ctx) == IFEMGPU_OK || fail("preprocessB");
  }

  bool assembleSystem(const TimeDomain&, const Vectors&, bool = true, bool = false) override
  {
    return ifemgpu_assemble(ctx, 1) == IFEMGPU_OK || fail("assembleSystem");
  }

  bool solveSystem(Vector& solution, int, double*, const char* = "displacement",
                   size_t = 0) override
  {
    ifemgpu_sizes sz{};
    if (ifemgpu_get_sizes(ctx, &sz) != IFEMGPU_OK) return fail("solveSystem");
    std::vector<double> x(sz.neq);
    ifemgpu_solve_info info{};
    if (ifemgpu_solve(ctx, &solver, x.data(), &info) != IFEMGPU_OK) return fail("solveSystem");
    solution.resize(sz.ndof);  // SAM::expandSolution: DOF order, fixed DOFs 0
    return ifemgpu_expand_solution(ctx, x.data(), solution.ptr(), 1.0) == IFEMGPU_OK ||
           fail("solveSystem");
  }

  //! \brief The GPU context (for the other entry points of include/ifemgpu.h).
  ifemgpu_ctx* gpu() const { return ctx; }

protected:
  bool fail(const char* method, const char* what = nullptr) const
  {
    std::cerr << " *** GpuSIM3D::" << method << ": "
              << (what ? what : ctx ? ifemgpu_last_error(ctx) : "no GPU context") << std::endl;
    return false;
  }

private:
  struct FaceBC { int patch, face, dofs; double value; };
  struct FaceLoad { int patch, face; double t[3]; };
  ifemgpu_ctx* ctx = nullptr;
  ifemgpu_material material{IFEMGPU_ELASTICITY, 0.0, 0.0, 0, 1.0, 0.3, {0.0, 0.0, 0.0}};
  ifemgpu_solver_options solver{};
  std::vector<FaceBC> faceBCs;
  std::vector<FaceLoad> faceLoads;
};

#endif  // IFEMGPU_ADAPTER_GPUSIM3D_H
