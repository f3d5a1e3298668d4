/*
 * hala_gb.hpp — C++ host layer of the GB300 sparse Krylov path, over the C ABI in hgb.h.
 *
 * Recreates, in namespace hala, the GPU-engine surface the reference's solvers and users call
 * for this path, with the same names and argument meaning:
 *   gpu_engine            gpu/hala_gpu_engine.hpp:47      (device, stream)
 *   gpu_vector<T>         gpu/hala_gpu_vector.hpp:49      (RAII device vector, load / unload)
 *   make_sparse_matrix    gpu/hala_cuda_sparse_general.hpp:383-401 -> gpu_sparse_matrix<T>::gemv
 *   sparse_gemv           gpu/hala_cuda_sparse_general.hpp:408-419
 *   make_ilu / ilu_apply  gpu/hala_gpu_ilu.hpp:54-192, wax/hala_sparse_extensions.hpp:51-105
 *   make_triangular_matrix / sparse_trsv   gpu/hala_cuda_sparse_triangular.hpp:38-421
 *   dot / norm2 / axpy / scal / vcopy / set_zero   gpu/hala_gpu_blas1.hpp, engine.hpp:336
 *   stop_criteria         hex/solvers/hala_solvers_core.hpp:52-70
 *   solve_cg / solve_cg_ilu / solve_gmres_ilu   hex/solvers/hala_solvers_cg.hpp, _gmres.hpp
 *   solve_batch_cg_ilu                          hex/solvers/hala_solvers_cg_batch.hpp
 *   mixed_engine          wax/hala_lib_extensions.hpp:68 (host vectors in, device compute)
 * Errors throw std::runtime_error carrying the library message, as the reference's check_cuda()
 * does (gpu/hala_cuda_common.hpp:78-152).  Header only; link with -lhgb -lcudart.
 */
#ifndef HALA_GB_HPP
#define HALA_GB_HPP

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../hgb.h"

namespace hala {

inline void hgb_check(int status, const char *what) {
    if (status != HGB_OK)
        throw std::runtime_error(std::string("hala::") + what + ": " + hgb_last_error());
}
inline void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("hala::") + what + ": " + cudaGetErrorString(e));
}

template <typename T> struct hgb_type;
template <> struct hgb_type<double> { static constexpr hgb_dtype value = HGB_F64; };
template <> struct hgb_type<float> { static constexpr hgb_dtype value = HGB_F32; };

/* ------------------------------------------------------------------------ engine -------- */
class gpu_engine {
public:
    explicit gpu_engine(int device = 0) : dev(device) {
        hgb_ctx *c = nullptr;
        hgb_check(hgb_ctx_create(device, &c), "gpu_engine");
        ctx = std::shared_ptr<hgb_ctx>(c, [](hgb_ctx *p) { hgb_ctx_destroy(p); });
    }
    int device() const { return dev; }
    void set_stream(cudaStream_t s) const { hgb_check(hgb_ctx_set_stream(ctx.get(), (void *)s), "set_stream"); }
    void synchronize() const { hgb_check(hgb_ctx_synchronize(ctx.get()), "synchronize"); }
    hgb_ctx *handle() const { return ctx.get(); }

private:
    int dev;
    std::shared_ptr<hgb_ctx> ctx;
};

/* ------------------------------------------------------------------------ vectors ------- */
template <typename T>
class gpu_vector {
public:
    using value_type = T;
    gpu_vector() = default;
    explicit gpu_vector(size_t n, int device = 0) : dev(device) { resize(n); }
    gpu_vector(gpu_vector const &) = delete;
    gpu_vector &operator=(gpu_vector const &) = delete;
    gpu_vector(gpu_vector &&o) noexcept : dev(o.dev), num(o.num), ptr(o.ptr) { o.ptr = nullptr; o.num = 0; }
    gpu_vector &operator=(gpu_vector &&o) noexcept {
        std::swap(dev, o.dev); std::swap(num, o.num); std::swap(ptr, o.ptr);
        return *this;
    }
    ~gpu_vector() { if (ptr) cudaFree(ptr); }

    void resize(size_t n) {
        if (n == num) return;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        num = n;
        if (n) cuda_check(cudaMalloc(&ptr, sizeof(T) * n), "gpu_vector");
    }
    size_t size() const { return num; }
    T *data() { return ptr; }
    T const *data() const { return ptr; }
    int device() const { return dev; }

    template <class Host> void load(Host const &h) {
        resize(h.size());
        if (num) cuda_check(cudaMemcpy(ptr, h.data(), sizeof(T) * num, cudaMemcpyHostToDevice), "load");
    }
    template <class Host> void unload(Host &h) const {
        h.resize(num);
        if (num) cuda_check(cudaMemcpy(h.data(), ptr, sizeof(T) * num, cudaMemcpyDeviceToHost), "unload");
    }
    std::vector<T> unload() const { std::vector<T> h; unload(h); return h; }

private:
    int dev = 0;
    size_t num = 0;
    T *ptr = nullptr;
};

template <typename T>
gpu_vector<T> make_gpu_vector(std::vector<T> const &h, int device = 0) {
    gpu_vector<T> v(0, device);
    v.load(h);
    return v;
}

/* gpu_engine::load(cpu vector) -> gpu_vector (engine.hpp) */
template <typename T>
gpu_vector<T> load(gpu_engine const &e, std::vector<T> const &h) {
    gpu_vector<T> v(0, e.device());
    v.load(h);
    return v;
}

/* new_vector(engine, x): an uninitialised vector of the same type and size */
template <typename T>
gpu_vector<T> new_vector(gpu_engine const &e, gpu_vector<T> const &x) { return gpu_vector<T>(x.size(), e.device()); }

/* ------------------------------------------------------------------------ BLAS-1 -------- */
inline double dot(gpu_engine const &e, gpu_vector<double> const &x, gpu_vector<double> const &y) {
    double r = 0; hgb_check(hgb_dot_f64(e.handle(), (int)x.size(), x.data(), y.data(), &r, 0), "dot"); return r;
}
inline float dot(gpu_engine const &e, gpu_vector<float> const &x, gpu_vector<float> const &y) {
    float r = 0; hgb_check(hgb_dot_f32(e.handle(), (int)x.size(), x.data(), y.data(), &r, 0), "dot"); return r;
}
inline double norm2(gpu_engine const &e, gpu_vector<double> const &x) {
    double r = 0; hgb_check(hgb_nrm2_f64(e.handle(), (int)x.size(), x.data(), &r, 0), "norm2"); return r;
}
inline float norm2(gpu_engine const &e, gpu_vector<float> const &x) {
    float r = 0; hgb_check(hgb_nrm2_f32(e.handle(), (int)x.size(), x.data(), &r, 0), "norm2"); return r;
}
template <typename FS>
void axpy(gpu_engine const &e, FS alpha, gpu_vector<double> const &x, gpu_vector<double> &y) {
    hgb_check(hgb_axpy_f64(e.handle(), (int)x.size(), (double)alpha, x.data(), y.data()), "axpy");
}
template <typename FS>
void axpy(gpu_engine const &e, FS alpha, gpu_vector<float> const &x, gpu_vector<float> &y) {
    hgb_check(hgb_axpy_f32(e.handle(), (int)x.size(), (float)alpha, x.data(), y.data()), "axpy");
}
template <typename FS>
void scal(gpu_engine const &e, FS alpha, gpu_vector<double> &x) {
    hgb_check(hgb_scal_f64(e.handle(), (int)x.size(), (double)alpha, x.data()), "scal");
}
template <typename FS>
void scal(gpu_engine const &e, FS alpha, gpu_vector<float> &x) {
    hgb_check(hgb_scal_f32(e.handle(), (int)x.size(), (float)alpha, x.data()), "scal");
}
template <typename T>
void vcopy(gpu_engine const &e, gpu_vector<T> const &x, gpu_vector<T> &y) {
    y.resize(x.size());
    if (std::is_same<T, double>::value)
        hgb_check(hgb_copy_f64(e.handle(), (int)x.size(), (double const *)x.data(), (double *)y.data()), "vcopy");
    else
        hgb_check(hgb_copy_f32(e.handle(), (int)x.size(), (float const *)x.data(), (float *)y.data()), "vcopy");
}
template <typename T>
void set_zero(gpu_engine const &e, gpu_vector<T> &x) {
    hgb_check(hgb_set_zero(e.handle(), sizeof(T) * x.size(), x.data()), "set_zero");
}

/* ------------------------------------------------------------------- sparse matrix ------ */
template <typename T>
class gpu_sparse_matrix {
public:
    using value_type = T;
    using engine_type = gpu_engine;
    gpu_sparse_matrix(gpu_engine const &e, int rows, int cols, int nnz, int const *pntr, int const *indx,
                      T const *vals)
        : eng(e), nrows(rows), ncols(cols) {
        hgb_csr *A = nullptr;
        hgb_check(hgb_csr_create(e.handle(), rows, cols, nnz, pntr, indx, vals, hgb_type<T>::value, &A), "make_sparse_matrix");
        h = std::shared_ptr<hgb_csr>(A, [](hgb_csr *p) { hgb_csr_destroy(p); });
    }
    /* gemv(trans, alpha, x, beta, y), general.hpp:265-277 */
    template <typename FA, typename FB>
    void gemv(char trans, FA alpha, gpu_vector<T> const &x, FB beta, gpu_vector<T> &y) const {
        size_t out = (trans == 'N' || trans == 'n') ? nrows : ncols;
        if (y.size() != out) y.resize(out);
        hgb_check(hgb_csr_gemv(h.get(), trans, (double)alpha, x.data(), (double)beta, y.data()), "gemv");
    }
    template <typename FA, typename FB, class Buff>
    void gemv(char trans, FA alpha, gpu_vector<T> const &x, FB beta, gpu_vector<T> &y, Buff &&) const {
        gemv(trans, alpha, x, beta, y);
    }
    /* the kernels need no workspace */
    template <typename FA, typename FB>
    size_t gemv_buffer_size(char, FA, gpu_vector<T> const &, FB, gpu_vector<T> &) const { return 0; }
    hgb_csr *handle() const { return h.get(); }
    int rows() const { return nrows; }
    int cols() const { return ncols; }

private:
    gpu_engine eng;
    int nrows, ncols;
    std::shared_ptr<hgb_csr> h;
};

template <typename T>
gpu_sparse_matrix<T> make_sparse_matrix(gpu_engine const &e, int num_rows, gpu_vector<int> const &pntr,
                                        gpu_vector<int> const &indx, gpu_vector<T> const &vals) {
    return gpu_sparse_matrix<T>(e, num_rows, num_rows, (int)indx.size(), pntr.data(), indx.data(), vals.data());
}

/* sparse_gemv(gpu_engine, trans, M, N, alpha, pntr, indx, vals, x, beta, y) */
template <typename FA, typename FB>
void sparse_gemv(gpu_engine const &e, char trans, int M, int N, FA alpha, gpu_vector<int> const &pntr,
                 gpu_vector<int> const &indx, gpu_vector<double> const &vals, gpu_vector<double> const &x, FB beta,
                 gpu_vector<double> &y) {
    size_t out = (trans == 'N' || trans == 'n') ? M : N;
    if (y.size() != out) y.resize(out);
    hgb_check(hgb_spmv_f64(e.handle(), trans, M, N, (int)indx.size(), pntr.data(), indx.data(), vals.data(),
                           (double)alpha, x.data(), (double)beta, y.data()), "sparse_gemv");
}
template <typename FA, typename FB>
void sparse_gemv(gpu_engine const &e, char trans, int M, int N, FA alpha, gpu_vector<int> const &pntr,
                 gpu_vector<int> const &indx, gpu_vector<float> const &vals, gpu_vector<float> const &x, FB beta,
                 gpu_vector<float> &y) {
    size_t out = (trans == 'N' || trans == 'n') ? M : N;
    if (y.size() != out) y.resize(out);
    hgb_check(hgb_spmv_f32(e.handle(), trans, M, N, (int)indx.size(), pntr.data(), indx.data(), vals.data(),
                           (float)alpha, x.data(), (float)beta, y.data()), "sparse_gemv");
}

/* --------------------------------------------------------------------------- ILU -------- */
template <typename T>
class gpu_ilu {
public:
    using value_type = T;
    using engine_type = gpu_engine;
    gpu_ilu(gpu_engine const &e, gpu_vector<int> const &pntr, gpu_vector<int> const &indx, gpu_vector<T> const &vals,
            char policy)
        : eng(e), n((int)pntr.size() - 1) {
        hgb_ilu *M = nullptr;
        int st = hgb_ilu0_create(e.handle(), n, (int)indx.size(), pntr.data(), indx.data(), vals.data(),
                                 hgb_type<T>::value, hgb_type<T>::value, policy, &M);
        if (st != HGB_OK && st != HGB_ERR_ZERO_PIVOT) hgb_check(st, "make_ilu");
        h = std::shared_ptr<hgb_ilu>(M, [](hgb_ilu *p) { hgb_ilu0_destroy(p); });
    }
    /* apply(x, r, num_rhs[, temp]), gpu_ilu.hpp:150-173 */
    void apply(gpu_vector<T> const &x, gpu_vector<T> &r, int num_rhs = 1) const {
        if (num_rhs != 1) throw std::runtime_error("hala::gpu_ilu::apply: one right-hand side");
        if (r.size() != (size_t)n) r.resize(n);
        hgb_check(hgb_ilu0_apply(h.get(), 'N', x.data(), r.data()), "ilu apply");
    }
    template <class Buff>
    void apply(gpu_vector<T> const &x, gpu_vector<T> &r, int num_rhs, Buff &&) const { apply(x, r, num_rhs); }
    size_t buffer_size(gpu_vector<T> const &, gpu_vector<T> const &, int) const { return 0; }
    gpu_vector<T> get_temp_buffer(gpu_vector<T> const &, gpu_vector<T> const &, int) const { return gpu_vector<T>(); }
    gpu_engine const &engine() const { return eng; }
    hgb_ilu *handle() const { return h.get(); }

private:
    gpu_engine eng;
    int n;
    std::shared_ptr<hgb_ilu> h;
};

template <typename T>
gpu_ilu<T> make_ilu(gpu_engine const &e, gpu_vector<int> const &pntr, gpu_vector<int> const &indx,
                    gpu_vector<T> const &vals, char policy = 'N') {
    return gpu_ilu<T>(e, pntr, indx, vals, policy);
}
template <typename T>
void ilu_apply(gpu_ilu<T> const &ilu, gpu_vector<T> const &x, gpu_vector<T> &r, int num_rhs = 1) { ilu.apply(x, r, num_rhs); }
template <typename T, class Buff>
void ilu_apply(gpu_ilu<T> const &ilu, gpu_vector<T> const &x, gpu_vector<T> &r, int num_rhs, Buff &&) { ilu.apply(x, r, num_rhs); }
template <typename T>
gpu_vector<T> ilu_temp_buffer(gpu_ilu<T> const &, gpu_vector<T> const &, gpu_vector<T> const &, int = 1) { return gpu_vector<T>(); }

/* ------------------------------------------------------------------ triangular ---------- */
template <typename T>
class gpu_triangular_matrix {
public:
    gpu_triangular_matrix(gpu_engine const &e, char uplo, char diag, gpu_vector<int> const &pntr,
                          gpu_vector<int> const &indx, gpu_vector<T> const &vals)
        : n((int)pntr.size() - 1) {
        hgb_tri *t = nullptr;
        hgb_check(hgb_tri_create(e.handle(), uplo, diag, n, (int)indx.size(), pntr.data(), indx.data(), vals.data(),
                                 hgb_type<T>::value, &t), "make_triangular_matrix");
        h = std::shared_ptr<hgb_tri>(t, [](hgb_tri *p) { hgb_tri_destroy(p); });
    }
    template <typename FA>
    void trsv(char trans, FA alpha, gpu_vector<T> const &b, gpu_vector<T> &x) const {
        if (x.size() != (size_t)n) x.resize(n);
        hgb_check(hgb_tri_solve(h.get(), trans, (double)alpha, b.data(), x.data()), "trsv");
    }

private:
    int n;
    std::shared_ptr<hgb_tri> h;
};
template <typename T>
gpu_triangular_matrix<T> make_triangular_matrix(gpu_engine const &e, char uplo, char diag, gpu_vector<int> const &pntr,
                                                gpu_vector<int> const &indx, gpu_vector<T> const &vals) {
    return gpu_triangular_matrix<T>(e, uplo, diag, pntr, indx, vals);
}
template <class Tri, typename FA, typename T>
void sparse_trsv(char trans, Tri const &tri, FA alpha, gpu_vector<T> const &b, gpu_vector<T> &x) {
    tri.trsv(trans, alpha, b, x);
}

/* ---------------------------------------------------------------------- solvers --------- */
template <typename precision>
struct stop_criteria {
    int max_iter;
    precision tol;
    stop_criteria(int max_iterations) : max_iter(max_iterations), tol(0) {}
    template <typename U, typename = std::enable_if_t<std::is_floating_point<U>::value>>
    stop_criteria(U tolerance) : max_iter(INT_MAX), tol((precision)tolerance) {}
    template <typename U>
    stop_criteria(U tolerance, int max_iterations) : max_iter(max_iterations), tol((precision)tolerance) {}
};

/* solve_cg_ilu(gpu_engine, stop, pntr, indx, vals, ilu, b, x): returns the iteration count */
template <typename T>
int solve_cg_ilu(gpu_engine const &e, stop_criteria<T> const &stop, gpu_vector<int> const &pntr,
                 gpu_vector<int> const &indx, gpu_vector<T> const &vals, gpu_ilu<T> const &ilu,
                 gpu_vector<T> const &b, gpu_vector<T> &x) {
    int n = (int)pntr.size() - 1;
    if (x.size() < (size_t)n) { x.resize(n); set_zero(e, x); }
    auto A = make_sparse_matrix(e, n, pntr, indx, vals);
    hgb_solve_info info{};
    hgb_check(hgb_cg_solve(e.handle(), A.handle(), ilu.handle(), b.data(), x.data(), (double)stop.tol, stop.max_iter,
                           &info), "solve_cg_ilu");
    return info.iterations;
}
template <typename T>
int solve_cg_ilu(gpu_engine const &e, stop_criteria<T> const &stop, gpu_vector<int> const &pntr,
                 gpu_vector<int> const &indx, gpu_vector<T> const &vals, gpu_vector<T> const &b, gpu_vector<T> &x,
                 char policy = 'N') {
    auto ilu = make_ilu(e, pntr, indx, vals, policy);
    return solve_cg_ilu(e, stop, pntr, indx, vals, ilu, b, x);
}
/* solve_cg without preconditioner */
template <typename T>
int solve_cg(gpu_engine const &e, stop_criteria<T> const &stop, gpu_vector<int> const &pntr,
             gpu_vector<int> const &indx, gpu_vector<T> const &vals, gpu_vector<T> const &b, gpu_vector<T> &x) {
    int n = (int)pntr.size() - 1;
    if (x.size() < (size_t)n) { x.resize(n); set_zero(e, x); }
    auto A = make_sparse_matrix(e, n, pntr, indx, vals);
    hgb_solve_info info{};
    hgb_check(hgb_cg_solve(e.handle(), A.handle(), nullptr, b.data(), x.data(), (double)stop.tol, stop.max_iter, &info),
              "solve_cg");
    return info.iterations;
}
/* solve_batch_cg_ilu(gpu_engine, stop, pntr, indx, vals, ilu, B, X), hex/solvers/hala_solvers_cg_batch.hpp:
 * B and X hold num_rhs = B.size() / n column-major right-hand sides */
template <typename T>
int solve_batch_cg_ilu(gpu_engine const &e, stop_criteria<T> const &stop, gpu_vector<int> const &pntr,
                       gpu_vector<int> const &indx, gpu_vector<T> const &vals, gpu_ilu<T> const &ilu,
                       gpu_vector<T> const &B, gpu_vector<T> &X) {
    int n = (int)pntr.size() - 1;
    int nrhs = (int)(B.size() / (size_t)n);
    if (X.size() < B.size()) { X.resize(B.size()); set_zero(e, X); }
    auto A = make_sparse_matrix(e, n, pntr, indx, vals);
    hgb_solve_info info{};
    hgb_check(hgb_cg_solve_nrhs(e.handle(), A.handle(), ilu.handle(), nrhs, B.data(), X.data(), (double)stop.tol,
                                stop.max_iter, &info), "solve_batch_cg_ilu");
    return info.iterations;
}
template <typename T>
int solve_batch_cg_ilu(gpu_engine const &e, stop_criteria<T> const &stop, gpu_vector<int> const &pntr,
                       gpu_vector<int> const &indx, gpu_vector<T> const &vals, gpu_vector<T> const &B,
                       gpu_vector<T> &X, char policy = 'N') {
    auto ilu = make_ilu(e, pntr, indx, vals, policy);
    return solve_batch_cg_ilu(e, stop, pntr, indx, vals, ilu, B, X);
}

/* solve_gmres_ilu(gpu_engine, stop, restart, pntr, indx, vals, ilu, b, x): double or float (the
 * reference's template, hex/solvers/hala_solvers_gmres.hpp:252-267); returns the applications */
template <typename T>
int solve_gmres_ilu(gpu_engine const &e, stop_criteria<T> const &stop, int restart, gpu_vector<int> const &pntr,
                    gpu_vector<int> const &indx, gpu_vector<T> const &vals, gpu_ilu<T> const &ilu,
                    gpu_vector<T> const &b, gpu_vector<T> &x) {
    int n = (int)pntr.size() - 1;
    if (x.size() < (size_t)n) { x.resize(n); set_zero(e, x); }
    auto A = make_sparse_matrix(e, n, pntr, indx, vals);
    hgb_solve_info info{};
    hgb_check(hgb_gmres_solve(e.handle(), A.handle(), ilu.handle(), restart, b.data(), x.data(), (double)stop.tol,
                              stop.max_iter, &info), "solve_gmres_ilu");
    return info.iterations;
}
template <typename T>
int solve_gmres_ilu(gpu_engine const &e, stop_criteria<T> const &stop, int restart, gpu_vector<int> const &pntr,
                    gpu_vector<int> const &indx, gpu_vector<T> const &vals, gpu_vector<T> const &b, gpu_vector<T> &x,
                    char policy = 'N') {
    auto ilu = make_ilu(e, pntr, indx, vals, policy);
    return solve_gmres_ilu(e, stop, restart, pntr, indx, vals, ilu, b, x);
}
/* solve_gmres without preconditioner (solve_gmres(engine, stop, restart, A, no preconditioner, b, x)) */
template <typename T>
int solve_gmres(gpu_engine const &e, stop_criteria<T> const &stop, int restart, gpu_vector<int> const &pntr,
                gpu_vector<int> const &indx, gpu_vector<T> const &vals, gpu_vector<T> const &b, gpu_vector<T> &x) {
    int n = (int)pntr.size() - 1;
    if (x.size() < (size_t)n) { x.resize(n); set_zero(e, x); }
    auto A = make_sparse_matrix(e, n, pntr, indx, vals);
    hgb_solve_info info{};
    hgb_check(hgb_gmres_solve(e.handle(), A.handle(), nullptr, restart, b.data(), x.data(), (double)stop.tol,
                              stop.max_iter, &info), "solve_gmres");
    return info.iterations;
}

/* --------------------------------------------------------------- mixed engine ----------- */
/* wax/hala_lib_extensions.hpp:68: CPU vectors in, GPU compute, x written back */
class mixed_engine {
public:
    explicit mixed_engine(int device = 0) : g(device) {}
    gpu_engine const &gpu() const { return g; }

private:
    gpu_engine g;
};

/* mixed_ilu: holds the device factor of a host matrix (wax/hala_lib_extensions.hpp:314-366) */
template <typename T>
class mixed_ilu {
public:
    mixed_ilu(mixed_engine const &e, std::vector<int> const &pntr, std::vector<int> const &indx,
              std::vector<T> const &vals, char policy = 'N')
        : p(load(e.gpu(), pntr)), i(load(e.gpu(), indx)), v(load(e.gpu(), vals)), f(e.gpu(), p, i, v, policy) {}
    gpu_ilu<T> const &cilu() const { return f; }

private:
    gpu_vector<int> p, i;
    gpu_vector<T> v;
    gpu_ilu<T> f;
};
template <typename T>
mixed_ilu<T> make_ilu(mixed_engine const &e, std::vector<int> const &pntr, std::vector<int> const &indx,
                      std::vector<T> const &vals, char policy = 'N') {
    return mixed_ilu<T>(e, pntr, indx, vals, policy);
}

/* solve_cg_ilu(mixed_engine, ...), hex/solvers/hala_solvers_cg.hpp:330-340 */
inline int solve_cg_ilu(mixed_engine const &e, stop_criteria<double> const &stop, std::vector<int> const &pntr,
                        std::vector<int> const &indx, std::vector<double> const &vals, mixed_ilu<double> const &ilu,
                        std::vector<double> const &b, std::vector<double> &x) {
    int n = (int)pntr.size() - 1;
    if (x.size() < (size_t)n) x.assign(n, 0.0);
    hgb_solve_info info{};
    hgb_check(hgb_mixed_cg_solve(e.gpu().handle(), n, (int)indx.size(), pntr.data(), indx.data(), vals.data(),
                                 ilu.cilu().handle(), b.data(), x.data(), stop.tol, stop.max_iter, &info),
              "solve_cg_ilu(mixed_engine)");
    return info.iterations;
}

}  // namespace hala

#endif
