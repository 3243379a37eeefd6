// A FoamAdapter-style heat-transfer solver written against the C++ façade
// (the shape of examples/heatTransfer/heatTransfer.cpp:60-83):
//   while (runTime.loop()) { T.oldTime() = T; solve(ddt(T) - laplacian(kappa, T)); }
// with the solver options of a mapped fvSolution entry in turn (Jacobi, ILU(0),
// BiCG, the ||b|| baseline, the multigrid solver), plus one explicit upwind
// advection step and the gradient of the result.  Writes the fields as raw
// little-endian doubles to the path given on the command line;
// tests/test_gpu_adapter.py compares them with the CPU oracle.
#include <cmath>
#include <cstdio>
#include <vector>

#include "fvgb_neon.hpp"

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: heat_adapter OUT.bin\n");
        return 2;
    }
    try {
        // mesh: 20 x 16 x 12 jittered box (the reference reads it from polyMesh)
        fvgb_box_spec spec{20, 16, 12, 1.0, 0.8, 0.6, 0.1, 12345ull, 0};
        int64_t sz[7];
        fvgb::check(fvgb_box_sizes(&spec, sz));
        const int32_t n = (int32_t)sz[2], nif = (int32_t)sz[3], nbf = (int32_t)sz[4], np = (int32_t)sz[5];
        std::vector<double> V(n), C(3 * n), Sf(3 * nif), Cf(3 * nif), magSf(nif), w(nif), dc(nif), bSf(3 * nbf),
            bCf(3 * nbf), bmagSf(nbf), bw(nbf), bdc(nbf);
        std::vector<int32_t> own(nif), nei(nif), bcells(nbf), poff(np + 1);
        fvgb_mesh_arrays a{nullptr, V.data(), C.data(), own.data(), nei.data(), Sf.data(), Cf.data(),
                           magSf.data(), w.data(), dc.data(), bcells.data(), bSf.data(), bCf.data(),
                           bmagSf.data(), bw.data(), bdc.data(), poff.data()};
        fvgb::check(fvgb_box_build(&spec, &a));
        fvgb_mesh_desc d{n, nif, nbf, np, V.data(), C.data(), own.data(), nei.data(), Sf.data(), magSf.data(),
                         w.data(), dc.data(), bcells.data(), bSf.data(), bmagSf.data(), bw.data(), bdc.data(),
                         poff.data()};
        fvgb::UnstructuredMesh mesh(d);

        // kappa per cell -> face conductivity by linear interpolation
        std::vector<double> k(n);
        for (int32_t c = 0; c < n; ++c) k[c] = 1.0 + 0.5 * std::sin(0.37 * c);
        std::vector<fvgb::PatchBC> zg(np, fvgb::PatchBC::zeroGradient());
        fvgb::VolumeField kappa(mesh, "kappa", k, zg);
        fvgb::SurfaceField kappaf(mesh);
        fvgb::SurfaceInterpolation(mesh, "linear").interpolate(kappa, kappaf);

        std::vector<fvgb::PatchBC> tbc(np, fvgb::PatchBC::zeroGradient());
        tbc[0] = fvgb::PatchBC::fixedValue({400.0});
        fvgb::VolumeField T(mesh, "T", std::vector<double>(n, 300.0), tbc);
        fvgb::DeviceArray<double> Told(n);
        std::FILE* f = std::fopen(argv[1], "wb");
        if (!f) return 4;
        auto put = [&](const fvgb::DeviceArray<double>& arr) {
            std::vector<double> h = arr.copyToHost();
            std::fwrite(h.data(), sizeof(double), h.size(), f);
        };
        fvgb::SolverConfig cfg;
        cfg.relTol = 1e-8;
        auto steps = [&](int count, const char* what) -> bool {
            for (int step = 0; step < count; ++step) {
                Told.copyFrom(T.internalVector());
                fvgb::PDESolver eqn(fvgb::dsl::imp::ddt(Told) - fvgb::dsl::imp::laplacian(kappaf), T, 0.01);
                fvgb::SolverStats st = eqn.solve(cfg);
                std::printf("%s step %d: initial residual %.6e final %.6e iterations %d\n", what, step,
                            st.initResNorm, st.finalResNorm, st.numIter);
                if (st.status != FVGB_OK) return false;
            }
            return true;
        };
        // the solver options of a mapped fvSolution entry, one after another:
        // PCG + DIC, PCG + DILU (ILU(0)), PBiCG, a ResidualNorm with the ||b||
        // baseline; the field after each phase goes to the output
        if (!steps(3, "CG+Jacobi")) return 3;
        put(T.internalVector());
        cfg.ilu = true;
        if (!steps(2, "CG+ILU")) return 3;
        put(T.internalVector());
        cfg.ilu = false;
        cfg.bicg = true;
        if (!steps(1, "BiCG")) return 3;
        put(T.internalVector());
        cfg.bicg = false;
        cfg.rhsBaseline = true;
        cfg.relTol = 1e-6;
        if (!steps(1, "CG, ||b|| baseline")) return 3;
        put(T.internalVector());
        // explicit upwind advection of T with a uniform velocity (1, 0.5, 0.25)
        std::vector<double> U(3 * n), Ub(3 * nbf);
        for (int32_t c = 0; c < n; ++c) U[3 * c] = 1.0, U[3 * c + 1] = 0.5, U[3 * c + 2] = 0.25;
        for (int32_t b = 0; b < nbf; ++b) Ub[3 * b] = 1.0, Ub[3 * b + 1] = 0.5, Ub[3 * b + 2] = 0.25;
        fvgb::DeviceArray<double> dU(U), dUb(Ub);
        fvgb::SurfaceField phi(mesh);
        fvgb::flux(mesh, dU, dUb, phi);
        fvgb::DeviceArray<double> divT(n);
        fvgb::GaussGreenDiv(mesh, "upwind").div(divT, phi, T, 1.0);
        fvgb::DeviceArray<double> gradT(3 * (size_t)n);
        fvgb::GaussGreenGrad(mesh).grad(T, 1.0, gradT);
        fvgb::check_cuda(cudaDeviceSynchronize(), "sync");
        put(divT);
        put(gradT);
        // GAMG (the multigrid solver) for one more step
        cfg.rhsBaseline = false;
        cfg.relTol = 1e-8;
        cfg.multigridSolver = true;
        if (!steps(1, "multigrid solver")) return 3;
        put(T.internalVector());
        std::fclose(f);
        std::printf("ok %d cells\n", n);
    } catch (const fvgb::Error& e) {
        std::fprintf(stderr, "fvgb error: %s\n", e.what());
        return 1;
    }
    return 0;
}
