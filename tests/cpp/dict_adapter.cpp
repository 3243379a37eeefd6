// The C++ façade's dictionary calls used the way FoamAdapter uses NeoN's:
// the checks of the reference's test/test_readDict.cpp and
// test/test_compatibility.cpp, on the reference's case files (the directory
// they were unpacked to is argv[1]).  Host code only: no GPU is touched.
#include <cstdio>
#include <string>

#include "fvgb_neon.hpp"

static int failures = 0;
#define REQUIRE(c)                                                  \
    do {                                                            \
        if (!(c)) {                                                 \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
            ++failures;                                             \
        }                                                           \
    } while (0)

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string root = argv[1];
    try {
        // test_readDict.cpp:67-91
        fvgb::Dictionary t = fvgb::readFoamDictionary(root + "/test/setup_operator/system/testDictionary");
        REQUIRE(t.get<int64_t>("label") == 1);
        REQUIRE(t.get<double>("scalar") == 2.1);
        REQUIRE(t.get<double>("scalar2") == 2.0);
        REQUIRE(t.get<int>("scalarWriteAnsInt") == 2);
        REQUIRE((t.get<fvgb::Vec3>("vector") == fvgb::Vec3{1.0, 2.0, 3.0}));
        REQUIRE(t.get<std::string>("word") == "word");
        fvgb::Dictionary sub = t.subDict("subDict");
        REQUIRE(sub.get<double>("subScalar") == 4.1);
        REQUIRE((sub.get<fvgb::Vec3>("subVector") == fvgb::Vec3{5.0, 6.0, 7.0}));
        REQUIRE(sub.get<std::string>("subWord") == "subWord");
        // test_readDict.cpp:40-65
        fvgb::Dictionary fs = fvgb::readFoamDictionary(root + "/test/setup_operator/system/fvSchemes");
        REQUIRE(fs.subDict("ddtSchemes").get<std::string>("ddt(T)") == "Euler");
        fvgb::TokenList lim = fs.subDict("gradSchemes").get<fvgb::TokenList>("limited");
        REQUIRE(lim.size() == 4);
        REQUIRE(lim[0].text == "cellLimited" && lim[1].text == "Gauss" && lim[2].text == "linear");
        REQUIRE(lim[3].kind == FVGB_TOK_LABEL && lim[3].label == 1);
        fvgb::TokenList gU = fs.subDict("gradSchemes").get<fvgb::TokenList>("grad(U)");
        REQUIRE(gU.size() == 2 && gU[0].text == "Gauss" && gU[1].text == "linear");
        REQUIRE(fvgb::scheme(fs, "divSchemes", "div(phi,T)") == FVGB_SCHEME_LINEAR);
        // test_compatibility.cpp:38-85
        fvgb::Dictionary fv = fvgb::readFoamDictionary(root + "/test/setup_compatibility/system/fvSolution");
        fvgb::Dictionary solverDict = fv.subDict("solvers");
        fvgb::Dictionary solver1 = solverDict.subDict("solver1");
        const char* names[][2] = {{"PCG", "solver::Cg"}, {"PBiCG", "solver::Bicg"}, {"PBiCGStab", "solver::Bicgstab"}};
        for (auto& n : names) {
            fvgb::Dictionary s = solver1;  // a view: changes land in fv
            s.insert("solver", std::string(n[0]));
            fvgb::updateSolver(s);
            REQUIRE(s.get<std::string>("solver") == "Ginkgo");
            REQUIRE(s.get<std::string>("type") == n[1]);
        }
        solver1.insert("preconditioner", std::string("DIC"));
        fvgb::updatePreconditioner(solver1);
        REQUIRE(solver1.subDict("preconditioner").get<std::string>("type") == "preconditioner::Jacobi");
        REQUIRE(solver1.subDict("preconditioner").get<int>("max_block_size") == 1);
        solver1.insert("preconditioner", std::string("DILU"));
        fvgb::updatePreconditioner(solver1);
        fvgb::Dictionary pre = solver1.subDict("preconditioner");
        REQUIRE(pre.get<std::string>("type") == "preconditioner::Ilu");
        REQUIRE(pre.get<bool>("reverse_apply") == false);
        REQUIRE(pre.subDict("factorization").get<std::string>("type") == "factorization::ParIlu");
        // neoIcoFoam.cpp:38-42: map p, then configure the solve from it
        fvgb::Dictionary cav = fvgb::readFoamDictionary(root + "/tutorials/cavity/system/fvSolution");
        fvgb::Dictionary p = fvgb::mapFvSolution(cav.subDict("solvers").subDict("p"));
        REQUIRE(cav.subDict("solvers").subDict("p").get<std::string>("solver") == "PCG");
        REQUIRE(p.get<std::string>("solver") == "Ginkgo");
        fvgb::SolverConfig c = fvgb::solverConfig(p);
        REQUIRE(c.tolerance == 1e-6 && c.relTol == 0.0 && c.maxIter == 1000 && !c.bicgstab && !c.mixedPrecision);
        fvgb::Dictionary owned = p;  // an owned copy is independent
        owned.remove("criteria");
        REQUIRE(p.contains("criteria") && !owned.contains("criteria"));
        // GAMG -> the multigrid solver; PBiCG -> BiCG
        fvgb::SolverConfig mg = fvgb::solverConfig(fvgb::mapFvSolution(fvgb::Dictionary::parse("solver GAMG;")));
        REQUIRE(mg.multigridSolver && mg.method() == FVGB_SOLVER_MULTIGRID && !mg.multigrid);
        fvgb::SolverConfig bg =
            fvgb::solverConfig(fvgb::mapFvSolution(fvgb::Dictionary::parse("solver PBiCG; preconditioner DIC;")));
        REQUIRE(bg.bicg && bg.method() == FVGB_SOLVER_BICG);
        // DILU -> Ginkgo's Ilu with a ParIlu factorization: the ILU(0) preconditioner
        fvgb::SolverConfig il =
            fvgb::solverConfig(fvgb::mapFvSolution(fvgb::Dictionary::parse("solver PBiCGStab; preconditioner DILU;")));
        REQUIRE(il.ilu && il.bicgstab && !il.multigrid);
        bool threw = false;
        try {  // BiCG with ILU is not built
            fvgb::solverConfig(fvgb::mapFvSolution(fvgb::Dictionary::parse("solver PBiCG; preconditioner DILU;")));
        } catch (const fvgb::Error& e) {
            threw = e.status == FVGB_ERR_UNSUPPORTED;
        }
        REQUIRE(threw);
    } catch (const std::exception& e) {
        std::printf("exception: %s\n", e.what());
        return 1;
    }
    std::printf("%d failures\n", failures);
    return failures ? 1 : 0;
}

// compile check of the fvSolution-driven solve (not run here: it needs a GPU)
[[maybe_unused]] static fvgb::SolverStats solve_from_case(fvgb::PDESolver& eqn, const fvgb::Dictionary& fv) {
    return fvgb::solve(eqn, fv);
}
