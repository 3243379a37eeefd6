// fvgb_neon.hpp -- C++ façade over the fvgb C ABI with the names and argument
// meaning of the NeoN / FoamAdapter calls on the finite-volume hot path.
//
// A FoamAdapter solver written against NeoN, e.g. examples/heatTransfer/
// heatTransfer.cpp:67-76 or examples/neoIcoFoam/neoIcoFoam.cpp:94-166, switches
// to the GB300 path by replacing NeoN::finiteVolume::cellCentred /
// NeoN::dsl / FoamAdapter calls with the same-named ones below:
//   GaussGreenDiv(mesh, "upwind").div(out, phi, T, coeff)
//   GaussGreenGrad(mesh).grad(T, coeff, out)
//   GaussGreenLaplacian(mesh).laplacian(out, gamma, T, coeff)
//   SurfaceInterpolation(mesh, "linear").interpolate(src, dst)
//   FaceNormalGradient(mesh).faceNormalGrad(T, out)
//   PDESolver(dsl::imp::ddt(T) - dsl::imp::laplacian(gamma, T), T, dt).solve()
//   computeRAUandHByA, constrainHbyA, flux, updateFaceVelocity, updateVelocity
//   readFoamDictionary(path), mapFvSolution(dict), solverConfig(dict)
// Errors are C++ exceptions (fvgb::Error), as NeoN reports them; fields own
// device storage (RAII), operators borrow the mesh, outputs are caller-owned
// and accumulated into with a coefficient.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "fvgb.h"

namespace fvgb {

struct Error : std::runtime_error {
    fvgb_status status;
    Error(fvgb_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(fvgb_status s) {
    if (s != FVGB_OK) throw Error(s, std::string(fvgb_status_string(s)) + ": " + fvgb_last_error());
}

inline void check_cuda(cudaError_t e, const char* where) {
    if (e != cudaSuccess) throw Error(FVGB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Device array with value semantics for moves only.
template <class T>
class DeviceArray {
public:
    DeviceArray() = default;
    explicit DeviceArray(size_t n) : n_(n) {
        check_cuda(cudaMalloc(&p_, sizeof(T) * (n ? n : 1)), "cudaMalloc");
        check_cuda(cudaMemset(p_, 0, sizeof(T) * (n ? n : 1)), "cudaMemset");
    }
    DeviceArray(const std::vector<T>& h) : DeviceArray(h.size()) { upload(h); }
    DeviceArray(DeviceArray&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr, o.n_ = 0; }
    DeviceArray& operator=(DeviceArray&& o) noexcept {
        std::swap(p_, o.p_);
        std::swap(n_, o.n_);
        return *this;
    }
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    ~DeviceArray() {
        if (p_) cudaFree(p_);
    }
    void upload(const std::vector<T>& h) {
        if (h.size() != n_) throw Error(FVGB_ERR_INVALID_ARG, "DeviceArray::upload: size mismatch");
        check_cuda(cudaMemcpy(p_, h.data(), sizeof(T) * n_, cudaMemcpyHostToDevice), "upload");
    }
    std::vector<T> copyToHost() const {
        std::vector<T> h(n_);
        check_cuda(cudaMemcpy(h.data(), p_, sizeof(T) * n_, cudaMemcpyDeviceToHost), "copyToHost");
        return h;
    }
    void copyFrom(const DeviceArray& o, cudaStream_t s = nullptr) {
        check_cuda(cudaMemcpyAsync(p_, o.p_, sizeof(T) * n_, cudaMemcpyDeviceToDevice, s), "copy");
    }
    T* data() { return p_; }
    const T* data() const { return p_; }
    size_t size() const { return n_; }

private:
    T* p_ = nullptr;
    size_t n_ = 0;
};

// NeoN::UnstructuredMesh + BoundaryMesh on the device (meshAdapter.cpp:59-136).
class UnstructuredMesh {
public:
    explicit UnstructuredMesh(const fvgb_mesh_desc& d) : desc_(d) {
        fvgb_mesh* m = nullptr;
        check(fvgb_mesh_create(&d, &m));
        h_.reset(m);
        patch_offsets_.assign(d.patch_offsets, d.patch_offsets + d.n_patches + 1);
    }
    fvgb_mesh* handle() const { return h_.get(); }
    int32_t nCells() const { return desc_.n_cells; }
    int32_t nInternalFaces() const { return desc_.n_ifaces; }
    int32_t nBoundaryFaces() const { return desc_.n_bfaces; }
    int32_t nFaces() const { return desc_.n_ifaces + desc_.n_bfaces; }
    int32_t nBoundaries() const { return desc_.n_patches; }
    const std::vector<int32_t>& patchOffsets() const { return patch_offsets_; }

private:
    struct Del {
        void operator()(fvgb_mesh* m) const { fvgb_mesh_destroy(m); }
    };
    fvgb_mesh_desc desc_;
    std::unique_ptr<fvgb_mesh, Del> h_;
    std::vector<int32_t> patch_offsets_;
};

// A boundary condition of one patch (readers.hpp:43-95 mapping).
struct PatchBC {
    fvgb_bc_type type = FVGB_BC_CALCULATED;
    std::vector<double> value;  // one value (per component) or one per face (per component)
    static PatchBC fixedValue(std::vector<double> v) { return {FVGB_BC_FIXED_VALUE, std::move(v)}; }
    static PatchBC fixedGradient(std::vector<double> g) { return {FVGB_BC_FIXED_GRADIENT, std::move(g)}; }
    static PatchBC zeroGradient(int ncomp = 1) { return {FVGB_BC_FIXED_GRADIENT, std::vector<double>(ncomp, 0.0)}; }
    static PatchBC noSlip(int ncomp = 3) { return {FVGB_BC_FIXED_VALUE, std::vector<double>(ncomp, 0.0)}; }
    static PatchBC calculated() { return {FVGB_BC_CALCULATED, {}}; }
};

// VolumeField<scalar> (ncomp 1) or VolumeField<Vec3> (ncomp 3).
class VolumeField {
public:
    VolumeField(const UnstructuredMesh& mesh, std::string name, const std::vector<double>& internal,
                const std::vector<PatchBC>& bcs, int ncomp = 1)
        : mesh_(&mesh), name(std::move(name)), ncomp_(ncomp), internal_(internal),
          boundary_(size_t(mesh.nBoundaryFaces()) * ncomp) {
        if (internal.size() != size_t(mesh.nCells()) * ncomp)
            throw Error(FVGB_ERR_INVALID_ARG, "VolumeField: internal size mismatch");
        if (bcs.size() != size_t(mesh.nBoundaries()))
            throw Error(FVGB_ERR_INVALID_ARG, "VolumeField: one boundary condition per non-empty patch");
        std::vector<double> ref(size_t(mesh.nBoundaryFaces()) * ncomp, 0.0);
        const auto& off = mesh.patchOffsets();
        for (size_t p = 0; p < bcs.size(); ++p) {
            types_.push_back(bcs[p].type);
            const auto& v = bcs[p].value;
            const int32_t nfp = off[p + 1] - off[p];
            for (int32_t f = 0; f < nfp; ++f)
                for (int k = 0; k < ncomp; ++k) {
                    double x = 0.0;
                    if (v.size() == size_t(ncomp)) x = v[k];
                    else if (v.size() == size_t(nfp) * ncomp) x = v[size_t(f) * ncomp + k];
                    else if (v.size() == 1) x = v[0];
                    ref[size_t(off[p] + f) * ncomp + k] = x;
                }
        }
        ref_ = DeviceArray<double>(ref);
        correctBoundaryConditions();
    }
    void correctBoundaryConditions(cudaStream_t s = nullptr) {
        fvgb_bc bc = bc_struct();
        check(fvgb_bc_correct(mesh_->handle(), ncomp_, &bc, internal_.data(), boundary_.data(), s));
    }
    fvgb_bc bc_struct() const { return fvgb_bc{types_.data(), ref_.data()}; }
    DeviceArray<double>& internalVector() { return internal_; }
    const DeviceArray<double>& internalVector() const { return internal_; }
    DeviceArray<double>& boundaryValues() { return boundary_; }
    const DeviceArray<double>& boundaryValues() const { return boundary_; }
    const UnstructuredMesh& mesh() const { return *mesh_; }
    int ncomp() const { return ncomp_; }

private:
    const UnstructuredMesh* mesh_;

public:
    std::string name;

private:
    int ncomp_;
    DeviceArray<double> internal_, boundary_, ref_;
    std::vector<int32_t> types_;
};

class SurfaceField {
public:
    SurfaceField(const UnstructuredMesh& mesh, int ncomp = 1)
        : mesh_(&mesh), ncomp_(ncomp), values_(size_t(mesh.nFaces()) * ncomp) {}
    SurfaceField(const UnstructuredMesh& mesh, const std::vector<double>& v, int ncomp = 1)
        : mesh_(&mesh), ncomp_(ncomp), values_(v) {}
    DeviceArray<double>& internalVector() { return values_; }
    const DeviceArray<double>& internalVector() const { return values_; }
    int ncomp() const { return ncomp_; }

private:
    const UnstructuredMesh* mesh_;
    int ncomp_;
    DeviceArray<double> values_;
};

inline fvgb_scheme scheme_of(const std::string& s) {
    if (s == "linear") return FVGB_SCHEME_LINEAR;
    if (s == "upwind") return FVGB_SCHEME_UPWIND;
    throw Error(FVGB_ERR_UNSUPPORTED, "unknown interpolation scheme " + s);
}

class SurfaceInterpolation {
public:
    SurfaceInterpolation(const UnstructuredMesh& m, const std::string& scheme) : m_(m), s_(scheme_of(scheme)) {}
    void interpolate(const VolumeField& src, SurfaceField& dst, const SurfaceField* flux = nullptr,
                     cudaStream_t st = nullptr) const {
        if (s_ == FVGB_SCHEME_LINEAR)
            check(fvgb_interp_linear(m_.handle(), src.ncomp(), src.internalVector().data(),
                                     src.boundaryValues().data(), dst.internalVector().data(), st));
        else if (flux)
            check(fvgb_interp_upwind(m_.handle(), src.ncomp(), flux->internalVector().data(),
                                     src.internalVector().data(), src.boundaryValues().data(),
                                     dst.internalVector().data(), st));
        else
            throw Error(FVGB_ERR_INVALID_ARG, "upwind interpolation needs the face flux");
    }

private:
    const UnstructuredMesh& m_;
    fvgb_scheme s_;
};

class GaussGreenDiv {
public:
    GaussGreenDiv(const UnstructuredMesh& m, const std::string& scheme) : m_(m), s_(scheme_of(scheme)) {}
    void div(DeviceArray<double>& out, const SurfaceField& faceFlux, const VolumeField& phi, double coeff = 1.0,
             cudaStream_t st = nullptr) const {
        check(fvgb_div_explicit(m_.handle(), s_, phi.ncomp(), faceFlux.internalVector().data(),
                                phi.internalVector().data(), phi.boundaryValues().data(), coeff, out.data(), st));
    }

private:
    const UnstructuredMesh& m_;
    fvgb_scheme s_;
};

class GaussGreenGrad {
public:
    explicit GaussGreenGrad(const UnstructuredMesh& m) : m_(m) {}
    void grad(const VolumeField& phi, double coeff, DeviceArray<double>& out, cudaStream_t st = nullptr) const {
        check(fvgb_grad(m_.handle(), phi.internalVector().data(), phi.boundaryValues().data(), coeff, out.data(),
                        st));
    }

private:
    const UnstructuredMesh& m_;
};

// snGrad correction of a scheme: "Gauss linear corrected" / "corrected" -> true,
// "Gauss linear uncorrected" / "uncorrected" -> false.
inline bool corrected_of(const std::string& scheme) {
    const bool has_un = scheme.find("uncorrected") != std::string::npos;
    if (!has_un && scheme.find("corrected") != std::string::npos) return true;
    if (has_un || scheme.empty() || scheme == "Gauss linear" || scheme == "linear") return false;
    throw Error(FVGB_ERR_UNSUPPORTED, "unknown snGrad scheme " + scheme);
}

class GaussGreenLaplacian {
public:
    explicit GaussGreenLaplacian(const UnstructuredMesh& m, const std::string& scheme = "Gauss linear uncorrected")
        : m_(m), corrected_(corrected_of(scheme)) {}
    void laplacian(DeviceArray<double>& out, const SurfaceField& gamma, const VolumeField& phi, double coeff = 1.0,
                   cudaStream_t st = nullptr) const {
        auto fn = corrected_ ? fvgb_laplacian_explicit_corrected : fvgb_laplacian_explicit;
        check(fn(m_.handle(), phi.ncomp(), gamma.internalVector().data(), phi.internalVector().data(),
                 phi.boundaryValues().data(), coeff, out.data(), st));
    }

private:
    const UnstructuredMesh& m_;
    bool corrected_;
};

class FaceNormalGradient {
public:
    explicit FaceNormalGradient(const UnstructuredMesh& m, const std::string& scheme = "uncorrected")
        : m_(m), corrected_(corrected_of(scheme)) {}
    void faceNormalGrad(const VolumeField& phi, SurfaceField& out, cudaStream_t st = nullptr) const {
        auto fn = corrected_ ? fvgb_sngrad_corrected : fvgb_sngrad;
        check(fn(m_.handle(), phi.internalVector().data(), phi.boundaryValues().data(), out.internalVector().data(),
                 st));
    }

private:
    const UnstructuredMesh& m_;
    bool corrected_;
};

// An OpenFOAM case mesh read from constant/polyMesh (ascii or binary); desc()
// feeds UnstructuredMesh, readField/write the case's field files.
class PolyMesh {
public:
    explicit PolyMesh(const std::string& dir) {
        fvgb_polymesh* p = nullptr;
        check(fvgb_polymesh_read(dir.c_str(), &p, &desc_));
        h_.reset(p);
    }
    const fvgb_mesh_desc& desc() const { return desc_; }
    fvgb_polymesh* handle() const { return h_.get(); }
    // internalField [n*ncomp] on the host (n: cells, or internal faces for a surface field)
    std::vector<double> readField(const std::string& path, int ncomp = 1, bool surface = false) const {
        const int32_t n = surface ? desc_.n_ifaces : desc_.n_cells;
        std::vector<double> v((size_t)n * ncomp);
        check(fvgb_field_read(path.c_str(), n, ncomp, v.data()));
        return v;
    }
    void write(const std::string& path, const std::string& object, int ncomp, const std::vector<double>& internal,
               const std::vector<double>& boundary, int flags = 0) const {
        check(fvgb_field_write(path.c_str(), object.c_str(), h_.get(), ncomp, internal.data(), boundary.data(),
                               flags));
    }

private:
    struct Free {
        void operator()(fvgb_polymesh* p) const { fvgb_polymesh_free(p); }
    };
    std::unique_ptr<fvgb_polymesh, Free> h_;
    fvgb_mesh_desc desc_{};
};

// ------------------------------------------------------------------- dsl
namespace dsl {

struct Expression {
    std::vector<fvgb_term> terms;
    Expression operator+(const Expression& o) const {
        Expression e = *this;
        e.terms.insert(e.terms.end(), o.terms.begin(), o.terms.end());
        return e;
    }
    Expression operator-(const Expression& o) const {
        Expression e = *this;
        for (fvgb_term t : o.terms) {
            t.coeff = -t.coeff;
            e.terms.push_back(t);
        }
        return e;
    }
    friend Expression operator*(double c, Expression e) {
        for (auto& t : e.terms) t.coeff *= c;
        return e;
    }
};

namespace imp {
// ddt(psi): `old` holds psi's old-time values (NeoN oldTime(psi)).
inline Expression ddt(const DeviceArray<double>& old) {
    return {{fvgb_term{FVGB_TERM_DDT, 0, 1.0, old.data(), nullptr}}};
}
inline Expression laplacian(const SurfaceField& gamma) {
    return {{fvgb_term{FVGB_TERM_LAPLACIAN, 0, 1.0, nullptr, gamma.internalVector().data()}}};
}
// laplacian(gamma, psi) with a scheme; "Gauss linear corrected" adds the
// non-orthogonal correction of psi's current values to the right-hand side.
inline Expression laplacian(const SurfaceField& gamma, const VolumeField& psi,
                            const std::string& scheme = "Gauss linear uncorrected") {
    if (!corrected_of(scheme)) return laplacian(gamma);
    return {{fvgb_term{FVGB_TERM_LAPLACIAN, FVGB_SCHEME_CORRECTED, 1.0, psi.internalVector().data(),
                       gamma.internalVector().data()}}};
}
inline Expression div(const SurfaceField& flux, const std::string& scheme = "linear") {
    return {{fvgb_term{FVGB_TERM_DIV, scheme_of(scheme), 1.0, nullptr, flux.internalVector().data()}}};
}
inline Expression source(double c, const DeviceArray<double>* s = nullptr) {
    return {{fvgb_term{FVGB_TERM_SOURCE, 0, c, s ? s->data() : nullptr, nullptr}}};
}
}  // namespace imp

namespace exp {
// exp::div(phi) of a face flux, volume integrated into the right-hand side.
inline Expression div(const SurfaceField& flux) {
    return {{fvgb_term{FVGB_TERM_DIV_FLUX, 0, 1.0, nullptr, flux.internalVector().data()}}};
}
// any precomputed volume-integrated explicit contribution
inline Expression source(const DeviceArray<double>& e) {
    return {{fvgb_term{FVGB_TERM_EXPLICIT, 0, 1.0, e.data(), nullptr}}};
}
}  // namespace exp
}  // namespace dsl

struct SolverStats {
    double initResNorm = 0, finalResNorm = 0;
    int numIter = 0, numOuter = 0;
    fvgb_status status = FVGB_OK;
};

// fvSolution entries mapped as FoamAdapter maps them (fvSolution.cpp:106-142).
struct SolverConfig {
    double relTol = 0.0;
    double tolerance = 0.0;
    int maxIter = 1000;
    bool mixedPrecision = false;
    double innerRelTol = 0.0;  // 0: 0.1 for CG, 0.01 for BiCGStab (the fastest measured)
    int innerMaxIter = 1000;
    int maxOuter = 50;
    bool bicgstab = false;  // solver "BiCGStab" (fvSolution.cpp:25-26) instead of "CG"
    bool bicg = false;      // solver "BiCG" (PBiCG, fvSolution.cpp:24; FP64)
    bool multigridSolver = false;  // solver "Multigrid" on its own (GAMG, fvSolution.cpp:27)
    bool multigrid = false; // preconditioner solver::Multigrid instead of Jacobi (CG; with
                            // mixedPrecision the V-cycle runs in FP32 inside the FP64 CG)
    bool rhsBaseline = false;  // relTol relative to ||b|| (Ginkgo ResidualNorm, baseline rhs_norm)
    bool ilu = false;          // preconditioner Ilu/ParIlu (DILU, fvSolution.cpp:56-63): exact ILU(0);
                               // CG or BiCGStab, FP64
    int method() const {
        return multigridSolver ? FVGB_SOLVER_MULTIGRID
                               : bicg ? FVGB_SOLVER_BICG : bicgstab ? FVGB_SOLVER_BICGSTAB : FVGB_SOLVER_CG;
    }
};

class LinearSystem {
public:
    LinearSystem(const UnstructuredMesh& m, int ncomp = 1) : m_(m) {
        fvgb_ls* ls = nullptr;
        check(fvgb_ls_create(m.handle(), ncomp, &ls));
        h_.reset(ls);
    }
    fvgb_ls* handle() const { return h_.get(); }

private:
    struct Del {
        void operator()(fvgb_ls* l) const { fvgb_ls_destroy(l); }
    };
    const UnstructuredMesh& m_;
    std::unique_ptr<fvgb_ls, Del> h_;
};

// FoamAdapter::PDESolver (expression.hpp:23-179).
class PDESolver {
public:
    PDESolver(dsl::Expression expr, VolumeField& psi, double dt)
        : expr_(std::move(expr)), psi_(psi), dt_(dt), ls_(psi.mesh(), psi.ncomp()) {}
    LinearSystem& assemble(cudaStream_t st = nullptr) {
        fvgb_bc bc = psi_.bc_struct();
        check(fvgb_assemble(ls_.handle(), expr_.terms.data(), (int32_t)expr_.terms.size(), dt_, &bc,
                            psi_.boundaryValues().data(), st));
        return ls_;
    }
    void setReference(int32_t cell, double value) {
        needRef_ = true;
        refCell_ = cell;
        refValue_ = value;
    }
    SolverStats solve(const SolverConfig& c = {}, cudaStream_t st = nullptr) {
        assemble(st);
        if (needRef_) check(fvgb_set_reference(ls_.handle(), refCell_, refValue_, st));
        fvgb_solver_cfg cfg{c.relTol, c.tolerance, c.maxIter,
                            c.mixedPrecision ? FVGB_PREC_MIXED_IR : FVGB_PREC_FP64,
                            c.innerRelTol > 0 ? c.innerRelTol : (c.bicgstab ? 0.01 : 0.1),
                            c.innerMaxIter, c.maxOuter, 0, c.rhsBaseline ? FVGB_SOLVE_RHS_BASELINE : 0,
                            c.method(),
                            c.multigrid ? FVGB_PRECOND_MULTIGRID : c.ilu ? FVGB_PRECOND_ILU : FVGB_PRECOND_JACOBI};
        fvgb_solver_stats s{};
        fvgb_status r = fvgb_solve(ls_.handle(), psi_.internalVector().data(), &cfg, &s, st);
        if (r != FVGB_OK && r != FVGB_ERR_NOT_CONVERGED) check(r);  // non-convergence is not an error
        psi_.correctBoundaryConditions(st);
        return SolverStats{s.init_res_norm, s.final_res_norm, s.num_iter, s.num_outer, (fvgb_status)s.status};
    }
    LinearSystem& linearSystem() { return ls_; }
    VolumeField& getField() { return psi_; }

private:
    dsl::Expression expr_;
    VolumeField& psi_;
    double dt_;
    LinearSystem ls_;
    bool needRef_ = false;
    int32_t refCell_ = 0;
    double refValue_ = 0.0;
};

// ------------------------------------------- pressureVelocityCoupling.cpp:14-267
inline void computeRAUandHByA(PDESolver& UEqn, DeviceArray<double>& rAU, DeviceArray<double>& HbyA,
                              cudaStream_t st = nullptr) {
    check(fvgb_piso_rau_hbya(UEqn.linearSystem().handle(), UEqn.getField().internalVector().data(), rAU.data(),
                             HbyA.data(), st));
}
inline void constrainHbyA(const UnstructuredMesh& m, const std::vector<int32_t>& assignable,
                          const VolumeField& U, DeviceArray<double>& HbyA_b, cudaStream_t st = nullptr) {
    check(fvgb_piso_constrain_hbya(m.handle(), assignable.data(), U.boundaryValues().data(), HbyA_b.data(), st));
}
inline void flux(const UnstructuredMesh& m, const DeviceArray<double>& U, const DeviceArray<double>& U_b,
                 SurfaceField& out, cudaStream_t st = nullptr) {
    check(fvgb_flux_vec(m.handle(), U.data(), U_b.data(), out.internalVector().data(), st));
}
inline void updateFaceVelocity(const SurfaceField& predictedPhi, PDESolver& pEqn, SurfaceField& phi,
                               cudaStream_t st = nullptr) {
    check(fvgb_piso_face_update(pEqn.linearSystem().handle(), predictedPhi.internalVector().data(),
                                pEqn.getField().internalVector().data(), phi.internalVector().data(), st));
}
inline void updateVelocity(const UnstructuredMesh& m, const DeviceArray<double>& HbyA, const DeviceArray<double>& rAU,
                           const VolumeField& p, VolumeField& U, cudaStream_t st = nullptr) {
    check(fvgb_piso_velocity_update(m.handle(), HbyA.data(), rAU.data(), p.internalVector().data(),
                                    p.boundaryValues().data(), U.internalVector().data(), st));
}

// ------------------------------------------------ NeoN::Dictionary (host)
// FoamAdapter::convert(Foam::dictionary) (src/auxiliary/foamDictionary.cpp:
// 68-91, convert.cpp:17-45) over libfvgb's dictionary reader: get<T> gives a
// label (int64_t / int) for one integer token, a scalar (double) for one
// number, a word (std::string) for one word or quoted string, a Vec3 for
// (x y z), a bool for yes/no/on/off/true/false, the TokenList for anything
// else.  Copying an owned Dictionary copies its entries (NeoN::Dictionary has
// value semantics); subDict returns a view into its parent, as the reference's
// Dictionary& does, valid until that entry is replaced or removed.
using Vec3 = std::array<double, 3>;
struct Token {
    int32_t kind;  // FVGB_TOK_*
    std::string text;
    int64_t label;
    double scalar;
};
using TokenList = std::vector<Token>;

class Dictionary {
public:
    Dictionary() {
        check(fvgb_dict_create(&h_));
        owned_ = true;
    }
    static Dictionary read(const std::string& path) {
        fvgb_dict* d = nullptr;
        check(fvgb_dict_read(path.c_str(), &d));
        return Dictionary(d, true);
    }
    static Dictionary parse(const std::string& text, const std::string& includeDir = ".") {
        fvgb_dict* d = nullptr;
        check(fvgb_dict_parse(text.c_str(), includeDir.c_str(), &d));
        return Dictionary(d, true);
    }
    Dictionary(const Dictionary& o) : owned_(o.owned_) {
        if (o.owned_) check(fvgb_dict_copy(o.h_, &h_));
        else h_ = o.h_;
    }
    Dictionary& operator=(const Dictionary& o) {
        if (this != &o) {
            Dictionary t(o);
            std::swap(h_, t.h_);
            std::swap(owned_, t.owned_);
        }
        return *this;
    }
    Dictionary(Dictionary&& o) noexcept : h_(o.h_), owned_(o.owned_) { o.h_ = nullptr, o.owned_ = false; }
    ~Dictionary() {
        if (owned_ && h_) fvgb_dict_free(h_);
    }

    bool contains(const std::string& key) const { return fvgb_dict_find(h_, key.c_str()) >= 0; }
    bool isDict(const std::string& key) const { return fvgb_dict_sub(h_, at(key)) != nullptr; }
    Dictionary subDict(const std::string& key) const {
        fvgb_dict* s = fvgb_dict_sub(h_, at(key));
        if (!s) throw Error(FVGB_ERR_INVALID_ARG, "Dictionary::subDict: " + key + " is not a sub-dictionary");
        return Dictionary(s, false);
    }
    std::vector<std::string> keys() const {
        std::vector<std::string> k;
        for (int32_t i = 0; i < fvgb_dict_size(h_); ++i) k.emplace_back(fvgb_dict_key(h_, i));
        return k;
    }
    TokenList tokens(const std::string& key) const {
        const int32_t i = at(key);
        const int32_t n = fvgb_dict_ntokens(h_, i);
        if (n < 0) throw Error(FVGB_ERR_INVALID_ARG, "Dictionary: " + key + " is a sub-dictionary");
        TokenList t;
        for (int32_t j = 0; j < n; ++j) {
            Token k{};
            const char* txt = nullptr;
            check(fvgb_dict_token(h_, i, j, &k.kind, &txt, &k.label, &k.scalar));
            k.text = txt;
            t.push_back(k);
        }
        return t;
    }
    template <class T>
    T get(const std::string& key) const;

    void insert(const std::string& key, const std::string& word) {
        bool plain = !word.empty() && (std::isalpha((unsigned char)word[0]) || word[0] == '_');
        for (char c : word)
            if (std::isspace((unsigned char)c) || c == ';' || c == '{' || c == '}' || c == '(' || c == ')' ||
                c == '"' || c == '[' || c == ']')
                plain = false;
        check(fvgb_dict_set(h_, key.c_str(), (plain ? word : "\"" + word + "\"").c_str()));
    }
    void insert(const std::string& key, const char* word) { insert(key, std::string(word)); }
    void insert(const std::string& key, double v) {
        char b[64];
        std::snprintf(b, sizeof b, "%.17g", v);
        std::string t = b;
        if (t.find_first_of(".eEni") == std::string::npos) t += ".0";  // keep it a scalar token
        check(fvgb_dict_set(h_, key.c_str(), t.c_str()));
    }
    void insert(const std::string& key, int64_t v) { check(fvgb_dict_set(h_, key.c_str(), std::to_string(v).c_str())); }
    void insert(const std::string& key, int v) { insert(key, (int64_t)v); }
    void insert(const std::string& key, bool v) { check(fvgb_dict_set(h_, key.c_str(), v ? "true" : "false")); }
    void insert(const std::string& key, const Dictionary& d) { check(fvgb_dict_set_dict(h_, key.c_str(), d.h_, nullptr)); }
    void remove(const std::string& key) { check(fvgb_dict_remove(h_, key.c_str())); }
    fvgb_dict* handle() const { return h_; }

private:
    Dictionary(fvgb_dict* h, bool owned) : h_(h), owned_(owned) {}
    int32_t at(const std::string& key) const {
        const int32_t i = fvgb_dict_find(h_, key.c_str());
        if (i < 0) throw Error(FVGB_ERR_INVALID_ARG, "Dictionary: no entry " + key);
        return i;
    }
    const Token& single(const std::string& key, TokenList& t) const {
        t = tokens(key);
        if (t.size() != 1) throw Error(FVGB_ERR_INVALID_ARG, "Dictionary: " + key + " is not a single token");
        return t[0];
    }
    friend Dictionary mapFvSolution(const Dictionary&);
    fvgb_dict* h_ = nullptr;
    bool owned_ = false;
};

template <>
inline int64_t Dictionary::get<int64_t>(const std::string& key) const {
    TokenList t;
    const Token& k = single(key, t);
    if (k.kind != FVGB_TOK_LABEL) throw Error(FVGB_ERR_INVALID_ARG, "Dictionary: " + key + " is not a label");
    return k.label;
}
template <>
inline int Dictionary::get<int>(const std::string& key) const { return (int)get<int64_t>(key); }
template <>
inline double Dictionary::get<double>(const std::string& key) const {
    TokenList t;
    const Token& k = single(key, t);
    if (k.kind != FVGB_TOK_SCALAR && k.kind != FVGB_TOK_LABEL)
        throw Error(FVGB_ERR_INVALID_ARG, "Dictionary: " + key + " is not a number");
    return k.scalar;
}
template <>
inline std::string Dictionary::get<std::string>(const std::string& key) const {
    TokenList t;
    const Token& k = single(key, t);
    if (k.kind != FVGB_TOK_WORD && k.kind != FVGB_TOK_STRING)
        throw Error(FVGB_ERR_INVALID_ARG, "Dictionary: " + key + " is not a word");
    return k.text;
}
template <>
inline bool Dictionary::get<bool>(const std::string& key) const {
    const std::string w = get<std::string>(key);
    if (w == "yes" || w == "on" || w == "true") return true;
    if (w == "no" || w == "off" || w == "false" || w == "none") return false;
    throw Error(FVGB_ERR_INVALID_ARG, "Dictionary: " + key + " is not a switch");
}
template <>
inline Vec3 Dictionary::get<Vec3>(const std::string& key) const {
    const TokenList t = tokens(key);
    if (t.size() != 5 || t[0].text != "(" || t[4].text != ")")
        throw Error(FVGB_ERR_INVALID_ARG, "Dictionary: " + key + " is not a vector");
    Vec3 v{};
    for (int c = 0; c < 3; ++c) {
        if (t[c + 1].kind != FVGB_TOK_SCALAR && t[c + 1].kind != FVGB_TOK_LABEL)
            throw Error(FVGB_ERR_INVALID_ARG, "Dictionary: " + key + " is not a vector");
        v[c] = t[c + 1].scalar;
    }
    return v;
}
template <>
inline TokenList Dictionary::get<TokenList>(const std::string& key) const { return tokens(key); }

inline Dictionary readFoamDictionary(const std::string& path) { return Dictionary::read(path); }

// fvSolution.cpp:19-159
inline void updateSolver(Dictionary& d) { check(fvgb_fvsolution_update_solver(d.handle())); }
inline void updatePreconditioner(Dictionary& d) { check(fvgb_fvsolution_update_preconditioner(d.handle())); }
inline void updateCriteria(Dictionary& d) { check(fvgb_fvsolution_update_criteria(d.handle())); }
inline Dictionary mapFvSolution(const Dictionary& solverDict) {
    fvgb_dict* m = nullptr;
    check(fvgb_fvsolution_map(solverDict.handle(), &m));
    return Dictionary(m, true);
}
inline SolverConfig solverConfigOf(const fvgb_solver_cfg& c);
// A Ginkgo-form solver entry (mapFvSolution's output) as PDESolver::solve's
// configuration; an entry naming a configFile reads that Ginkgo JSON file,
// relative to configDir (the case's system directory).
inline SolverConfig solverConfig(const Dictionary& mapped, const std::string& configDir = "") {
    fvgb_solver_cfg c{};
    if (mapped.contains("configFile")) {
        if (configDir.empty()) throw Error(FVGB_ERR_INVALID_ARG, "solverConfig: configFile needs the case's system directory");
        check(fvgb_solver_cfg_from_json((configDir + "/" + mapped.get<std::string>("configFile")).c_str(), &c));
    } else {
        check(fvgb_solver_cfg_from_dict(mapped.handle(), &c));
    }
    return solverConfigOf(c);
}
inline SolverConfig solverConfigOf(const fvgb_solver_cfg& c) {
    SolverConfig s;
    s.relTol = c.rel_tol;
    s.tolerance = c.abs_tol;
    s.maxIter = c.max_iter;
    s.mixedPrecision = c.precision == FVGB_PREC_MIXED_IR;
    s.innerRelTol = c.inner_rel_tol;
    s.innerMaxIter = c.inner_max_iter;
    s.maxOuter = c.max_outer;
    s.bicgstab = c.method == FVGB_SOLVER_BICGSTAB;
    s.bicg = c.method == FVGB_SOLVER_BICG;
    s.multigridSolver = c.method == FVGB_SOLVER_MULTIGRID;
    s.multigrid = c.preconditioner == FVGB_PRECOND_MULTIGRID;
    s.rhsBaseline = (c.flags & FVGB_SOLVE_RHS_BASELINE) != 0;
    s.ilu = c.preconditioner == FVGB_PRECOND_ILU;
    return s;
}
// PDESolver::solve configured by the case's fvSolution as the reference reads
// it (expression.hpp:141-153): the entry solvers/<psi.name>; an entry in
// OpenFOAM form (solver PCG; ...) is mapped by mapFvSolution first.
inline SolverStats solve(PDESolver& eqn, const Dictionary& fvSolution, cudaStream_t st = nullptr) {
    Dictionary entry = fvSolution.subDict("solvers").subDict(eqn.getField().name);
    const bool ginkgo = entry.contains("solver") && entry.get<std::string>("solver") == "Ginkgo";
    return eqn.solve(solverConfig(ginkgo ? entry : mapFvSolution(entry)), st);
}
// The FVGB_SCHEME_* value fvSchemes gives `name` in `section` (own entry, else default).
inline int scheme(const Dictionary& fvSchemes, const std::string& section, const std::string& name) {
    int32_t s = 0;
    check(fvgb_scheme_from_dict(fvSchemes.handle(), section.c_str(), name.c_str(), &s));
    return s;
}

}  // namespace fvgb
