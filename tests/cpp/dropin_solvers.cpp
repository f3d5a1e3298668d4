// The reference's own solver templates over the GB300 backend (include/hala_gb/gpu/hala_gpu.hpp).
//
// Compiled with the reference's unmodified headers (common/ blas/ sparse/ lapack/ wax/ hex/) on the
// include path and include/hala_gb/gpu in place of the reference's gpu/ directory, with
// HALA_ENABLE_GPU and HALA_ENABLE_CUDA defined as the CUDA build defines them.  Nothing below is a
// solver of this repository: solve_cg_ilu, solve_gmres_ilu, solve_cg, solve_batch_cg_ilu and the
// mixed_engine overloads are the reference's templates (hex/solvers/hala_solvers_cg.hpp:181-369,
// hala_solvers_gmres.hpp:127-301, hala_solvers_cg_batch.hpp:68-248), instantiated on hala::gpu_engine
// and hala::mixed_engine, and every vector operation, product, ILU and triangular solve they
// resolve lands in libhgb.
//
// Run on a GPU machine it solves the reference's own test cases (tests/solvers_tests.hpp:13-55:
// the tridiagonal system whose ILU is exact, two CG iterations; the nonsymmetric 5 x 5 GMRES case)
// and a 3D anisotropic Poisson system against the host-side CG of the same templates, and prints
// one line per case.  Exit status 0 = all cases pass.
#include "hala.hpp"
#include "hala_solvers.hpp"

#include <cmath>
#include <csignal>
#include <cstdio>
#include <vector>

namespace {

int failures = 0;
void stage(const char *what) { std::printf("case: %s\n", what); }
void check(bool ok, const char *what) {
    std::printf("%s %s\n", ok ? "ok  " : "FAIL", what);
    if (!ok) failures++;
}
double rel_err(std::vector<double> const &a, std::vector<double> const &b) {
    double d = 0, n = 0;
    for (size_t i = 0; i < a.size(); i++) {
        d += (a[i] - b[i]) * (a[i] - b[i]);
        n += b[i] * b[i];
    }
    return std::sqrt(d / (n > 0 ? n : 1));
}

// 3D 7-point anisotropic operator on an m^3 grid, natural order (x fastest)
void aniso3d(int m, std::vector<int> &p, std::vector<int> &ix, std::vector<double> &v) {
    const double c[3] = {1.0, 1.0, 0.01};
    const int n = m * m * m;
    p.assign(1, 0);
    ix.clear();
    v.clear();
    for (int r = 0; r < n; r++) {
        const int x = r % m, y = (r / m) % m, z = r / (m * m);
        auto add = [&](int col, double val) { ix.push_back(col); v.push_back(val); };
        if (z > 0) add(r - m * m, -c[2]);
        if (y > 0) add(r - m, -c[1]);
        if (x > 0) add(r - 1, -c[0]);
        add(r, 2 * (c[0] + c[1] + c[2]));
        if (x < m - 1) add(r + 1, -c[0]);
        if (y < m - 1) add(r + m, -c[1]);
        if (z < m - 1) add(r + m * m, -c[2]);
        p.push_back((int)ix.size());
    }
}

}  // namespace

int main() {
    std::setvbuf(stdout, nullptr, _IONBF, 0);   // every line is out before anything can go wrong
    hala::gpu_engine engine(0);
    hala::mixed_engine mixed(engine);
    hala::cpu_engine cpu;

    {   // tests/solvers_tests.hpp:13-32: tridiagonal, exact ILU, two CG iterations from x0 = 0
        std::vector<int> p = {0, 2, 5, 8, 11, 13}, ix = {0, 1, 0, 1, 2, 1, 2, 3, 2, 3, 4, 3, 4};
        std::vector<double> v = {2, -1, -1, 2, -1, -1, 2, -1, -1, 2, -1, -1, 2};
        std::vector<double> b = {1, 0, 0, 0, 1}, xref = {1, 1, 1, 1, 1};
        std::vector<double> x;
        stage("tridiagonal, mixed_engine");
        int it = hala::solve_cg_ilu(mixed, hala::stop_criteria<double>(2), p, ix, v, b, x);
        check(it == 2 && rel_err(x, xref) < 1e-14, "solve_cg_ilu(mixed_engine): the exact tridiagonal case");
        auto gp = engine.load(p);
        auto gi = engine.load(ix);
        auto gv = engine.load(v);
        auto gb = engine.load(b);
        hala::gpu_vector<double> gx(engine.device());
        stage("tridiagonal, gpu_engine");
        it = hala::solve_cg_ilu(engine, hala::stop_criteria<double>(2), gp, gi, gv, gb, gx);
        check(it == 2 && rel_err(gx.unload(), xref) < 1e-14, "solve_cg_ilu(gpu_engine): the exact tridiagonal case");
    }
    {   // tests/solvers_tests.hpp:106-137: nonsymmetric 5 x 5, GMRES(3) with ILU
        std::vector<int> p = {0, 2, 5, 8, 11, 13}, ix = {0, 1, 0, 1, 2, 1, 2, 3, 2, 3, 4, 3, 4};
        std::vector<double> v = {4, -1, -2, 4, -1, -2, 4, -1, -2, 4, -1, -2, 4};
        std::vector<double> xref = {1, 2, 3, 4, 5}, b(5, 0.0);
        for (int r = 0; r < 5; r++)
            for (int k = p[r]; k < p[r + 1]; k++) b[r] += v[k] * xref[ix[k]];
        std::vector<double> x;
        stage("gmres 5x5, mixed_engine");
        hala::solve_gmres_ilu(mixed, hala::stop_criteria<double>(1e-12, 20), 3, p, ix, v, b, x);
        check(rel_err(x, xref) < 1e-10, "solve_gmres_ilu(mixed_engine): nonsymmetric 5 x 5");
    }
    {   // 3D anisotropic 12^3: the templates on gpu_engine against the same templates on cpu_engine
        std::vector<int> p, ix;
        std::vector<double> v;
        aniso3d(12, p, ix, v);
        const int n = (int)p.size() - 1;
        std::vector<double> xt(n), b(n, 0.0);
        for (int i = 0; i < n; i++) xt[i] = std::sin(0.37 * i);
        for (int r = 0; r < n; r++)
            for (int k = p[r]; k < p[r + 1]; k++) b[r] += v[k] * xt[ix[k]];
        double bn = 0;
        for (double t : b) bn += t * t;
        const double tol = 1e-10 * std::sqrt(bn);
        std::vector<double> xc;
        stage("12^3 cpu_engine");
        const int itc = hala::solve_cg_ilu(cpu, hala::stop_criteria<double>(tol), p, ix, v, b, xc);
        std::vector<double> xg;
        engine.set_spmv_mode("exact");
        stage("12^3 mixed_engine cg_ilu");
        const int itg = hala::solve_cg_ilu(mixed, hala::stop_criteria<double>(tol), p, ix, v, b, xg);
        check(std::abs(itg - itc) <= 1 + itc / 20 && rel_err(xg, xc) < 1e-8,
              "solve_cg_ilu(mixed_engine) vs cpu_engine, 12^3: iterations within 5%, solution within 1e-8");
        std::vector<double> xu;
        stage("12^3 mixed_engine cg");
        // the preconditioner of the mixed_engine overload receives gpu vectors
        // (hex/solvers/hala_solvers_core.hpp:97-100), so its copy names the GPU engine
        const int itu = hala::solve_cg(mixed, hala::stop_criteria<double>(tol), p, ix, v,
                                       [&](auto const &in, auto &out) { hala::vcopy(engine, in, out); }, b, xu);
        std::vector<double> xuc;
        const int itc2 = hala::solve_cg(cpu, hala::stop_criteria<double>(tol), p, ix, v,
                                        [](auto const &in, auto &out) { hala::vcopy(in, out); }, b, xuc);
        check(std::abs(itu - itc2) <= 1 + itc2 / 20 && rel_err(xu, xuc) < 1e-8,
              "solve_cg(mixed_engine) without preconditioner vs cpu_engine");
        std::vector<double> xgm;
        stage("12^3 mixed_engine gmres");
        const int itgm = hala::solve_gmres_ilu(mixed, hala::stop_criteria<double>(tol, 50), 30, p, ix, v, b, xgm);
        check(itgm > 0 && rel_err(xgm, xt) < 1e-7, "solve_gmres_ilu(mixed_engine), GMRES(30), 12^3");
        // several right-hand sides with one matrix: the reference's batch CG
        const int nrhs = 3;
        std::vector<double> B(hala::hala_size(n, nrhs)), X;
        for (int c = 0; c < nrhs; c++)
            for (int i = 0; i < n; i++) B[(size_t)c * n + i] = b[i] * (1.0 + c);
        stage("12^3 mixed_engine batch cg");
        const int itb = hala::solve_batch_cg_ilu(mixed, hala::stop_criteria<double>(tol * nrhs), p, ix, v, B, X);
        double e = 0;
        for (int c = 0; c < nrhs; c++) {
            std::vector<double> xc1(X.begin() + (size_t)c * n, X.begin() + (size_t)(c + 1) * n), xt1(n);
            for (int i = 0; i < n; i++) xt1[i] = xt[i] * (1.0 + c);
            e = std::max(e, rel_err(xc1, xt1));
        }
        check(itb > 0 && e < 1e-7, "solve_batch_cg_ilu(mixed_engine), three right-hand sides");
    }
    std::printf("%d failure(s)\n", failures);
    return failures ? 1 : 0;
}
