// C++ replay of the reference's sparse/solver test cases through include/hala_gb/hala_gb.hpp
// (tests/sparse_tests.hpp test_ilu, tests/solvers_tests.hpp test_cg, test_cg_batch and test_gmres,
// tests/cuda_sparse_tests.hpp sparse_matvec).  Exit code 0 when every check passes.
#include "hala_gb/hala_gb.hpp"

#include <cmath>
#include <cstdio>
#include <vector>

static int failures = 0;

static bool testvec(std::vector<double> const &x, std::vector<double> const &y, double corr = 1.0) {
    if (x.size() != y.size()) return false;
    double e = 0;
    for (size_t i = 0; i < x.size(); i++) {
        if (!std::isfinite(x[i])) return false;
        e += std::fabs(x[i] - y[i]);
    }
    return e / corr < 1e-14;
}

#define CHECK(c, name)                                              \
    do {                                                            \
        if (!(c)) { std::printf("FAIL %s\n", name); failures++; }   \
        else std::printf("ok   %s\n", name);                        \
    } while (0)

static std::vector<double> matvec(std::vector<int> const &p, std::vector<int> const &i,
                                  std::vector<double> const &v, std::vector<double> const &x) {
    std::vector<double> y(p.size() - 1, 0.0);
    for (size_t r = 0; r + 1 < p.size(); r++)
        for (int k = p[r]; k < p[r + 1]; k++) y[r] += v[k] * x[i[k]];
    return y;
}

int main() {
    hala::gpu_engine engine(0);
    using hala::gpu_vector;
    {   // sparse_matvec: y = 2 A x on the tridiagonal 5x5
        std::vector<int> pntr = {0, 2, 5, 8, 11, 13}, indx = {0, 1, 0, 1, 2, 1, 2, 3, 2, 3, 4, 3, 4};
        std::vector<double> vals = {2, 1, 1, 2, 1, 1, 2, 1, 1, 2, 1, 1, 2}, x = {1, 2, 3, 4, 5}, y;
        auto gp = hala::make_gpu_vector(pntr), gi = hala::make_gpu_vector(indx);
        auto gv = hala::make_gpu_vector(vals), gx = hala::make_gpu_vector(x);
        gpu_vector<double> gy;
        hala::sparse_gemv(engine, 'N', 5, 5, 2.0, gp, gi, gv, gx, 0.0, gy);
        gy.unload(y);
        auto ref = matvec(pntr, indx, vals, x);
        for (auto &r : ref) r *= 2;
        CHECK(testvec(y, ref), "sparse_matvec");
    }
    {   // test_ilu: 3x3 dense pattern
        std::vector<int> pntr = {0, 3, 6, 9}, indx = {0, 1, 2, 0, 1, 2, 0, 1, 2};
        std::vector<double> vals = {3, 2, 1, 2, 4, 3, 2, 1, 6}, x = {1, 2, 3}, r;
        auto gp = hala::make_gpu_vector(pntr), gi = hala::make_gpu_vector(indx);
        auto gv = hala::make_gpu_vector(vals);
        auto ilu = hala::make_ilu(engine, gp, gi, gv, 'N');
        gpu_vector<double> gr;
        hala::ilu_apply(ilu, hala::make_gpu_vector(x), gr);
        gr.unload(r);
        CHECK(testvec(r, {1.0 / 9.0, 1.0 / 9.0, 4.0 / 9.0}), "ilu apply");
    }
    std::vector<double> xref = {1, 2, 3, 4, 5};
    {   // test_cg: exact ILU on a tridiagonal matrix, stop_criteria(2)
        std::vector<int> pntr = {0, 2, 5, 8, 11, 13}, indx = {0, 1, 0, 1, 2, 1, 2, 3, 2, 3, 4, 3, 4};
        std::vector<double> vals = {2, 1, 1, 2, 1, 1, 2, 1, 1, 2, 1, 1, 2}, x;
        auto b = matvec(pntr, indx, vals, xref);
        auto gp = hala::make_gpu_vector(pntr), gi = hala::make_gpu_vector(indx);
        auto gv = hala::make_gpu_vector(vals);
        auto gb = hala::make_gpu_vector(b);
        auto ilu = hala::make_ilu(engine, gp, gi, gv, 'N');
        gpu_vector<double> gx;
        int it = hala::solve_cg_ilu(engine, hala::stop_criteria<double>(2), gp, gi, gv, ilu, gb, gx);
        gx.unload(x);
        CHECK(it == 2 && testvec(x, xref), "cg exact (2 iterations)");
        // gmres, exact case: restart 2, two restarts
        gpu_vector<double> gx2;
        hala::solve_gmres_ilu(engine, hala::stop_criteria<double>(2), 2, gp, gi, gv, ilu, gb, gx2);
        gx2.unload(x);
        CHECK(testvec(x, xref), "gmres exact");
    }
    {   // test_cg: cyclic 5x5 from x0, tol 1e-9, and the mixed engine
        std::vector<int> pntr = {0, 3, 6, 9, 12, 15}, indx = {0, 1, 4, 0, 1, 2, 1, 2, 3, 2, 3, 4, 0, 3, 4};
        std::vector<double> vals = {2, 1, 1, 1, 2, 1, 1, 2, 1, 1, 2, 1, 1, 1, 2}, x = {1, 3, -4, -7, 11};
        auto b = matvec(pntr, indx, vals, xref);
        auto gp = hala::make_gpu_vector(pntr), gi = hala::make_gpu_vector(indx);
        auto gv = hala::make_gpu_vector(vals);
        auto gx = hala::make_gpu_vector(x);
        hala::solve_cg_ilu(engine, hala::stop_criteria<double>(1e-9), gp, gi, gv, hala::make_gpu_vector(b), gx);
        gx.unload(x);
        double nrm = std::sqrt(55.0);
        CHECK(testvec(x, xref, nrm), "cg_ilu approximate");
        hala::mixed_engine mengine(0);
        auto milu = hala::make_ilu(mengine, pntr, indx, vals, 'N');
        std::vector<double> xm = {1, 3, -4, -7, 11};
        hala::solve_cg_ilu(mengine, hala::stop_criteria<double>(1e-9), pntr, indx, vals, milu, b, xm);
        CHECK(testvec(xm, xref, nrm), "cg_ilu mixed_engine");
    }
    {   // test_gmres: nonsymmetric 5x5, restart 6, tol 1e-9
        std::vector<int> pntr = {0, 2, 5, 8, 11, 12}, indx = {0, 1, 0, 1, 3, 1, 2, 3, 0, 2, 3, 4};
        std::vector<double> vals = {2, 1, 1, 3, 1, 1, 4, 1, 1, 1, 5, 2}, x;
        auto b = matvec(pntr, indx, vals, xref);
        auto gp = hala::make_gpu_vector(pntr), gi = hala::make_gpu_vector(indx);
        auto gv = hala::make_gpu_vector(vals);
        gpu_vector<double> gx;
        hala::solve_gmres_ilu(engine, hala::stop_criteria<double>(1e-9), 6, gp, gi, gv, hala::make_gpu_vector(b), gx);
        gx.unload(x);
        CHECK(testvec(x, xref), "gmres nonsymmetric");
        // the same system in float (the reference's template over float): the float tolerance
        std::vector<float> vf(vals.begin(), vals.end()), bf(b.begin(), b.end()), xf;
        gpu_vector<float> gxf;
        hala::solve_gmres_ilu(engine, hala::stop_criteria<float>(1e-5f), 6, gp, gi, hala::make_gpu_vector(vf),
                              hala::make_gpu_vector(bf), gxf);
        gxf.unload(xf);
        double ef = 0;
        for (size_t k = 0; k < xf.size(); k++) ef += std::fabs((double)xf[k] - xref[k]);
        CHECK(xf.size() == xref.size() && ef < 1e-4, "gmres nonsymmetric float");
    }
    {   // test_cg_batch: three right-hand sides, exact tridiagonal then cyclic with (1e-9, 6)
        std::vector<double> xb(15);
        for (int k = 0; k < 15; k++) xb[k] = k + 1;
        double nrm = 0;
        for (double v : xb) nrm += v * v;
        nrm = std::sqrt(nrm);
        auto block_b = [&](std::vector<int> const &p, std::vector<int> const &i, std::vector<double> const &v) {
            std::vector<double> b;
            for (int k = 0; k < 3; k++) {
                auto col = matvec(p, i, v, std::vector<double>(xb.begin() + 5 * k, xb.begin() + 5 * k + 5));
                b.insert(b.end(), col.begin(), col.end());
            }
            return b;
        };
        std::vector<int> pntr = {0, 2, 5, 8, 11, 13}, indx = {0, 1, 0, 1, 2, 1, 2, 3, 2, 3, 4, 3, 4};
        std::vector<double> vals = {2, 1, 1, 2, 1, 1, 2, 1, 1, 2, 1, 1, 2}, x;
        auto gp = hala::make_gpu_vector(pntr);
        auto gi = hala::make_gpu_vector(indx);
        auto gv = hala::make_gpu_vector(vals);
        auto ilu = hala::make_ilu(engine, gp, gi, gv, 'N');
        gpu_vector<double> gx;
        hala::solve_batch_cg_ilu(engine, hala::stop_criteria<double>(2), gp, gi, gv, ilu,
                                 hala::make_gpu_vector(block_b(pntr, indx, vals)), gx);
        gx.unload(x);
        CHECK(testvec(x, xb, nrm), "batch cg exact");
        pntr = {0, 3, 6, 9, 12, 15};
        indx = {0, 1, 4, 0, 1, 2, 1, 2, 3, 2, 3, 4, 0, 3, 4};
        vals = {2, 1, 1, 1, 2, 1, 1, 2, 1, 1, 2, 1, 1, 1, 2};
        auto cp = hala::make_gpu_vector(pntr);
        auto ci = hala::make_gpu_vector(indx);
        auto cv = hala::make_gpu_vector(vals);
        gpu_vector<double> gx2;
        hala::solve_batch_cg_ilu(engine, hala::stop_criteria<double>(1e-9, 6), cp, ci, cv,
                                 hala::make_gpu_vector(block_b(pntr, indx, vals)), gx2);
        gx2.unload(x);
        CHECK(testvec(x, xb, nrm), "batch cg_ilu approximate");
    }
    std::printf("%s\n", failures ? "HALA-GB CASES: FAIL" : "HALA-GB CASES: ALL PASS");
    return failures ? 1 : 0;
}
