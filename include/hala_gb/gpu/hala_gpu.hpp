/*
 * hala_gpu.hpp — the GB300 sparse Krylov path as a GPU backend of the reference's own templates.
 *
 * The reference's generic layers (common/, blas/, sparse/, wax/, hex/solvers/) reach their GPU
 * backend through `#include "hala_gpu.hpp"` (wax/hala_lib_extensions.hpp:17-19, under
 * HALA_ENABLE_GPU) and through unqualified overloads resolved on hala::gpu_engine and the GPU
 * vector types.  This header is a replacement for the reference's gpu/ directory: put
 * include/hala_gb/gpu on the include path instead of the reference's gpu/, define HALA_ENABLE_GPU
 * (and HALA_ENABLE_CUDA, as the CUDA build does), link libhgb and cudart.  The reference's solver
 * templates (solve_cg_core, solve_cg[_ilu], solve_gmres[_ilu], solve_batch_cg[_ilu], with
 * gpu_engine or mixed_engine) then run on the hand-written sm_103a kernels of libhgb instead of
 * cuSPARSE / cuBLAS.
 *
 * What it provides, each replacing the reference interface named beside it:
 *   gpu_engine                       gpu/hala_gpu_engine.hpp:47-300 (a shared hgb_ctx: device, stream)
 *   gpu_vector, gpu_wrapped_array    gpu/hala_gpu_vector.hpp:49-200, gpu/hala_gpu_wrap_array.hpp:30-120
 *   binded_gpu_vector, gpu_bind_vector   gpu/hala_gpu_vector.hpp:215-250, gpu/hala_gpu_engine.hpp:360
 *   new_vector, set_zero, gpu_pntr   gpu/hala_gpu_engine.hpp:320-420
 *   vcopy, norm2, dot, axpy, scal, iamax     gpu/hala_gpu_blas1.hpp, gpu/hala_gpu_overloads.hpp
 *   gemv (dense, tall-skinny)        gpu/hala_gpu_blas2.hpp:40 (GMRES krylov_project / _combine)
 *   dgmm, tbsv (diagonal)            gpu/hala_gpu_overloads.hpp (the batch_* column operations, vdivide)
 *   gpu_sparse_matrix, make_sparse_matrix, sparse_gemv, sparse_gemm   gpu/hala_cuda_sparse_general.hpp:192-441
 *   gpu_triangular_matrix, make_triangular_matrix                     gpu/hala_cuda_sparse_triangular.hpp:38-454
 *   gpu_ilu, make_ilu                gpu/hala_gpu_ilu.hpp:45-199
 * Real types (float, double) only.  Strided BLAS calls (inc != 1) throw std::runtime_error, as do
 * the dense BLAS-2/3 and LAPACK entries of the reference's gpu/ directory, which this path does
 * not replace (they are not declared here).  Errors throw std::runtime_error with the library's
 * message, as the reference's check_cuda() does (gpu/hala_cuda_common.hpp:78-152).
 *
 * Arithmetic: the sparse products run in the engine's SpMV mode (hgb_ctx_set_spmv_mode; the
 * default fuses multiply and add, gpu_engine::set_spmv_mode("exact") reproduces the reference's CPU
 * rounding bit for bit); ILU(0) factor and sweeps are bit-identical to the reference's CPU path.
 */
#ifndef HALA_GB_GPU_BACKEND_HPP
#define HALA_GB_GPU_BACKEND_HPP

#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <valarray>
#include <vector>

#include "../../hgb.h"

namespace hala {

/* ------------------------------------------------------------------ errors, devices --- */
inline void check_cuda(cudaError_t status, const char *function_name) {
    if (status != cudaSuccess)
        throw std::runtime_error(std::string(function_name) + " failed with message: " + cudaGetErrorString(status));
}
inline void check_hgb(int status, const char *function_name) {
    if (status != HGB_OK)
        throw std::runtime_error(std::string(function_name) + " failed with message: " + hgb_last_error());
}
inline int gpu_device_count() {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) return 0;
    return count;
}

template <typename T>
T *gpu_allocate(int gpu_device, size_t num_elements) {
    T *p = nullptr;
    check_cuda(cudaSetDevice(gpu_device), "cudaSetDevice()");
    if (num_elements) check_cuda(cudaMalloc((void **)&p, num_elements * sizeof(T)), "hala::gpu_allocate()");
    return p;
}
template <typename T>
void gpu_free(T *gpu_data) {
    if (gpu_data != nullptr) check_cuda(cudaFree((void *)gpu_data), "cudaFree()");
}

template <copy_direction dir, typename T>
void gpu_copy_n(T const *source, size_t num_entries, T *destination) {
    if (num_entries == 0) return;
    const cudaMemcpyKind kind = (dir == copy_direction::host2device)   ? cudaMemcpyHostToDevice
                                : (dir == copy_direction::device2host) ? cudaMemcpyDeviceToHost
                                                                       : cudaMemcpyDeviceToDevice;
    check_cuda(cudaMemcpy(destination, source, num_entries * sizeof(T), kind), "hala::gpu_copy_n()");
}

/* the path's element types: FP64 and FP32 (the reference's complex types are not implemented) */
template <typename T> struct hgb_real_type : std::false_type {};
template <> struct hgb_real_type<double> : std::true_type { static constexpr hgb_dtype dtype = HGB_F64; };
template <> struct hgb_real_type<float> : std::true_type { static constexpr hgb_dtype dtype = HGB_F32; };
template <typename T> void check_hgb_type() {
    static_assert(hgb_real_type<std::remove_cv_t<T>>::value || std::is_same<std::remove_cv_t<T>, int>::value,
                  "the GB300 backend holds float, double and int vectors");
}

/* --------------------------------------------------- wrapped arrays and vectors -------- */
template <typename ScalarType>
class gpu_wrapped_array {
public:
    using value_type = std::remove_const_t<ScalarType>;
    gpu_wrapped_array(ScalarType *arr, size_t num_entries) : gpu_data(arr), num(num_entries) {}
    gpu_wrapped_array(gpu_wrapped_array const &) = delete;
    void operator=(gpu_wrapped_array const &) = delete;
    gpu_wrapped_array(gpu_wrapped_array &&o) noexcept
        : gpu_data(std::exchange(o.gpu_data, nullptr)), num(std::exchange(o.num, 0)) {}
    void operator=(gpu_wrapped_array &&o) noexcept {
        std::swap(gpu_data, o.gpu_data);
        std::swap(num, o.num);
    }
    size_t size() const { return num; }
    ScalarType *data() { return gpu_data; }
    ScalarType const *data() const { return gpu_data; }
    template <class VectorLike> void load(VectorLike const &cpu_data) {
        if (num != (size_t)get_size(cpu_data)) throw std::runtime_error("hala::gpu_wrapped_array::load(): size mismatch");
        gpu_copy_n<copy_direction::host2device>(get_data(cpu_data), num, gpu_data);
    }
    template <class VectorLike> void unload(VectorLike &cpu_data) const {
        check_set_size(assume_output, cpu_data, num);
        gpu_copy_n<copy_direction::device2host>(gpu_data, num, get_data(cpu_data));
    }
    std::vector<value_type> unload() const {
        std::vector<value_type> h(num);
        unload(h);
        return h;
    }

private:
    ScalarType *gpu_data;
    size_t num;
};
template <typename ArrayType>
gpu_wrapped_array<ArrayType> wrap_gpu_array(ArrayType arr[], size_t num_entries) {
    return gpu_wrapped_array<ArrayType>(arr, num_entries);
}

/* RAII device vector: cudaMalloc / cudaFree (gpu/hala_gpu_vector.hpp:70-74,164) */
template <typename T>
class gpu_vector {
public:
    using value_type = T;
    gpu_vector(int deviceid = 0) : gpu(deviceid), num(0), gpu_data(nullptr) { check_hgb_type<T>(); }
    gpu_vector(size_t num_entries, int deviceid) : gpu(deviceid), num(0), gpu_data(nullptr) {
        check_hgb_type<T>();
        alloc(num_entries);
    }
    gpu_vector(gpu_vector const &o) : gpu(o.gpu), num(0), gpu_data(nullptr) {
        alloc(o.num);
        gpu_copy_n<copy_direction::device2device>(o.gpu_data, num, gpu_data);
    }
    gpu_vector(gpu_vector &&o) noexcept
        : gpu(o.gpu), num(std::exchange(o.num, 0)), gpu_data(std::exchange(o.gpu_data, nullptr)) {}
    ~gpu_vector() { clear(); }
    void operator=(gpu_vector const &o) {
        resize(o.num);
        gpu_copy_n<copy_direction::device2device>(o.gpu_data, num, gpu_data);
    }
    void operator=(gpu_vector &&o) noexcept {
        std::swap(gpu, o.gpu);
        std::swap(num, o.num);
        std::swap(gpu_data, o.gpu_data);
    }
    void clear() {
        gpu_free(gpu_data);
        gpu_data = nullptr;
        num = 0;
    }
    void resize(size_t new_size) {
        if (new_size == num) return;
        gpu_free(gpu_data);
        gpu_data = nullptr;
        alloc(new_size);
    }
    template <class VectorLike> void load(VectorLike const &cpu_data) {
        static_assert(std::is_same<T, typename define_type<VectorLike>::value_type>::value,
                      "mismatch in the type of gpu_vector and cpu_data when calling load()");
        resize(get_size(cpu_data));
        gpu_copy_n<copy_direction::host2device>(get_data(cpu_data), num, gpu_data);
    }
    template <class VectorLike> void unload(VectorLike &cpu_data) const {
        static_assert(std::is_same<T, typename define_type<VectorLike>::value_type>::value,
                      "mismatch in the type of gpu_vector and cpu_data when calling unload()");
        check_set_size(assume_output, cpu_data, num);
        gpu_copy_n<copy_direction::device2host>(gpu_data, num, get_data(cpu_data));
    }
    std::vector<T> unload() const {
        std::vector<T> h(num);
        unload(h);
        return h;
    }
    std::valarray<T> unload_valarray() const {
        std::valarray<T> h(num);
        unload(h);
        return h;
    }
    T *data() { return gpu_data; }
    T const *data() const { return gpu_data; }
    operator T *() { return gpu_data; }
    operator T const *() const { return gpu_data; }
    size_t size() const { return num; }
    int device() const { return gpu; }
    bool empty() const { return num == 0; }
    void fill(T value) {
        if (num == 0) return;
        if (value == T(0)) {
            check_cuda(cudaMemset(gpu_data, 0, num * sizeof(T)), "gpu_vector::fill()");
            return;
        }
        std::vector<T> h(num, value);
        gpu_copy_n<copy_direction::host2device>(h.data(), num, gpu_data);
    }

private:
    void alloc(size_t n) {
        num = n;
        gpu_data = gpu_allocate<T>(gpu, n);
    }
    int gpu;
    size_t num;
    T *gpu_data;
};

template <class VectorLike>
inline auto make_gpu_vector(VectorLike const &cpu_data, int gpuid = 0) {
    gpu_vector<typename define_type<VectorLike>::value_type> v(gpuid);
    v.load(cpu_data);
    return v;
}
template <typename T>
inline auto make_gpu_vector(size_t num_entries, int gpuid = 0) {
    return gpu_vector<T>(num_entries, gpuid);
}

template <typename T> struct deviceid_extractor<gpu_vector<T>> {
    static int device(gpu_vector<T> const &x) { return x.device(); }
};
template <typename T> struct deviceid_extractor<const gpu_vector<T>> {
    static int device(gpu_vector<T> const &x) { return x.device(); }
};

/* a device copy of a host vector, written back when it leaves scope (gpu/hala_gpu_vector.hpp:233) */
template <typename T, class VectorLike>
struct binded_gpu_vector {
    using value_type = T;
    binded_gpu_vector(int gpuid, VectorLike &v) : vec(v), cvec(gpuid) {
        static_assert(!std::is_const<VectorLike>::value, "Cannot bind to a const vector!");
        cvec.load(v);
    }
    ~binded_gpu_vector() { cvec.unload(vec); }
    T *data() { return cvec.data(); }
    T const *data() const { return cvec.data(); }
    void resize(size_t n) { cvec.resize(n); }
    size_t size() const { return cvec.size(); }
    int device() const { return cvec.device(); }

private:
    VectorLike &vec;
    gpu_vector<T> cvec;
};

/* ------------------------------------------------------------------------ engine ------- */
/* gpu/hala_gpu_engine.hpp:47: the device and stream the path runs on.  Copies share one context
 * (the reference's copies share its library handles). */
struct gpu_engine {
    gpu_engine(int deviceid = 0) : cgpu(deviceid) {
        hgb_ctx *c = nullptr;
        check_hgb(hgb_ctx_create(deviceid, &c), "hala::gpu_engine()");
        ctx = std::shared_ptr<hgb_ctx>(c, [](hgb_ctx *p) { hgb_ctx_destroy(p); });
    }
    gpu_engine(cudaStream_t streamid, int deviceid) : gpu_engine(deviceid) { set_stream(streamid); }
    gpu_engine(gpu_engine const &) = default;
    gpu_engine(gpu_engine &&) = default;
    gpu_engine &operator=(gpu_engine &&) = default;
    gpu_engine &operator=(gpu_engine const &) = default;

    int device() const { return cgpu; }
    void synchronize() const { check_hgb(hgb_ctx_synchronize(ctx.get()), "hala::gpu_engine::synchronize()"); }
    void set_stream(cudaStream_t streamid) const {
        check_hgb(hgb_ctx_set_stream(ctx.get(), (void *)streamid), "hala::gpu_engine::set_stream()");
    }
    void set_active_device() const { check_cuda(cudaSetDevice(cgpu), "cudaSetDevice()"); }
    /* "fused" (the default) or "exact" (the reference's separately rounded products) */
    void set_spmv_mode(std::string const &mode) const {
        check_hgb(hgb_ctx_set_spmv_mode(ctx.get(), mode == "exact" ? HGB_SPMV_EXACT : HGB_SPMV_FUSED),
                  "hala::gpu_engine::set_spmv_mode()");
    }
    hgb_ctx *handle() const { return ctx.get(); }

    template <class VectorLike> auto load(VectorLike const &cpu_data) const { return make_gpu_vector(cpu_data, cgpu); }
    template <class VectorLike> auto load(VectorLike const &cpu_data, size_t size) const {
        return make_gpu_vector(wrap_array(get_data(cpu_data), size), cgpu);
    }
    template <class VectorLike> auto unload(VectorLike const &gpu_data) const {
        std::vector<get_standard_type<VectorLike>> result(get_size(gpu_data));
        gpu_copy_n<copy_direction::device2host>(get_data(gpu_data), get_size(gpu_data), result.data());
        return result;
    }
    template <typename T> auto vector(size_t num_entries, T value) const {
        gpu_vector<T> x(num_entries, cgpu);
        x.fill(value);
        return x;
    }
    template <class vec> auto vcopy(vec const &x) const;
    template <typename T> auto wrap_array(T *array, size_t num_entries) const { return wrap_gpu_array(array, num_entries); }
    template <typename T> using dfvector = gpu_vector<T>;

    template <class one_gpu_vec> void check_gpu(one_gpu_vec const &x) const {
        const int d = get_device(x);
        if (d > -1 && d != cgpu) throw std::runtime_error("hala::gpu_engine: vector on another device");
    }
    template <class first_gpu_vec, class second_gpu_vec, class... other_gpu_vecs>
    void check_gpu(first_gpu_vec const &x, second_gpu_vec const &y, other_gpu_vecs const &...other) const {
        check_gpu(x);
        check_gpu(y, other...);
    }
    /* scalars of the BLAS-1 reductions are returned to the host (the reference's
     * CUBLAS_POINTER_MODE_HOST); the device-pointer mode is a no-op kept for signature parity */
    void set_blas_device_pntr() const {}
    void reset_blas_device_pntr() const {}

private:
    int cgpu;
    std::shared_ptr<hgb_ctx> ctx;
};

template <typename T> struct vector_constructor<gpu_vector<T>> {
    static auto make_one(gpu_engine const &engine) { return gpu_vector<T>(engine.device()); }
};

template <class VectorLike>
auto new_vector(gpu_engine const &engine, VectorLike const &) {
    return vector_constructor<get_vdefault<gpu_engine, VectorLike>>::make_one(engine);
}

template <class vec>
auto gpu_engine::vcopy(vec const &x) const {
    auto y = new_vector(*this, x);
    check_set_size(assume_output, y, get_size(x));
    gpu_copy_n<copy_direction::device2device>(get_standard_data(x), get_size(x), get_standard_data(y));
    return y;
}

/* set_zero(gpu_engine, n, x), gpu/hala_gpu_engine.hpp:336-352 (one memset here) */
template <class VectorLike>
void set_zero(gpu_engine const &engine, size_t num_entries, VectorLike &&x) {
    if (num_entries == 0) return;
    check_set_size(assume_output, x, num_entries);
    using T = get_standard_type<VectorLike>;
    check_hgb(hgb_set_zero(engine.handle(), num_entries * sizeof(T), (void *)get_standard_data(x)), "hala::set_zero()");
}

template <class VectorLike>
auto gpu_bind_vector(gpu_engine const &e, VectorLike &x) {
    return binded_gpu_vector<get_standard_type<VectorLike>, VectorLike>(e.device(), x);
}

template <typename ArrayType>
auto wrap_array(gpu_engine const &engine, ArrayType arr[], size_t num_entries) {
    return engine.wrap_array(arr, num_entries);
}

struct device_pntr {};
struct host_pntr {};
/* pointer-mode guard of the reference (gpu/hala_gpu_engine.hpp:395-445) */
template <typename pntr_mode>
struct gpu_pntr {
    static_assert(std::is_same<pntr_mode, device_pntr>::value || std::is_same<pntr_mode, host_pntr>::value,
                  "gpu_pntr can be used only with device_pntr and host_pntr pntr_mode types");
    explicit gpu_pntr(gpu_engine const &) {}
};

/* ------------------------------------------------------------------------ BLAS-1 ------- */
namespace hgb_detail {
inline void unit_stride(int inc, const char *what) {
    if (inc != 1) throw std::runtime_error(std::string("hala::") + what + ": the GB300 backend takes unit strides");
}
template <class V> inline auto ptr(V &&x) { return get_standard_data(x); }
}  // namespace hgb_detail

template <class VectorLikeX, class VectorLikeY>
inline void vcopy(gpu_engine const &engine, int N, VectorLikeX const &x, int incx, VectorLikeY &&y, int incy) {
    check_types(x, y);
    engine.check_gpu(x, y);
    hgb_detail::unit_stride(incx, "vcopy");
    hgb_detail::unit_stride(incy, "vcopy");
    check_set_size(assume_output, y, N);
    using T = get_standard_type<VectorLikeX>;
    if (N <= 0) return;
    if (std::is_same<T, double>::value)
        check_hgb(hgb_copy_f64(engine.handle(), N, (double const *)get_standard_data(x), (double *)get_standard_data(y)), "hala::vcopy()");
    else if (std::is_same<T, float>::value)
        check_hgb(hgb_copy_f32(engine.handle(), N, (float const *)get_standard_data(x), (float *)get_standard_data(y)), "hala::vcopy()");
    else
        gpu_copy_n<copy_direction::device2device>(get_standard_data(x), (size_t)N, get_standard_data(y));
}
template <class VectorLikeX, class VectorLikeY>
inline void vcopy(gpu_engine const &engine, VectorLikeX const &x, VectorLikeY &&y, int incx = 1, int incy = 1, int N = -1) {
    valid::default_size(x, incx, N);
    vcopy(engine, N, x, incx, y, incy);
}

template <class VectorLike>
auto norm2(gpu_engine const &engine, int N, VectorLike const &x, int incx) {
    check_types(x);
    engine.check_gpu(x);
    hgb_detail::unit_stride(incx, "norm2");
    using T = get_standard_type<VectorLike>;
    static_assert(hgb_real_type<T>::value, "hala::norm2 on the GB300 backend: float or double");
    T r = T(0);
    if (N <= 0) return r;
    if (std::is_same<T, double>::value)
        check_hgb(hgb_nrm2_f64(engine.handle(), N, (double const *)get_standard_data(x), (double *)&r, 0), "hala::norm2()");
    else
        check_hgb(hgb_nrm2_f32(engine.handle(), N, (float const *)get_standard_data(x), (float *)&r, 0), "hala::norm2()");
    return r;
}
template <class VectorLikeX>
inline auto norm2(gpu_engine const &engine, VectorLikeX const &x, int incx = 1, int N = -1) {
    valid::default_size(x, incx, N);
    return norm2(engine, N, x, incx);
}

template <bool conjugate = true, class VectorLikeX, class VectorLikeY>
auto dot(gpu_engine const &engine, int N, VectorLikeX const &x, int incx, VectorLikeY const &y, int incy) {
    check_types(x, y);
    engine.check_gpu(x, y);
    hgb_detail::unit_stride(incx, "dot");
    hgb_detail::unit_stride(incy, "dot");
    using T = get_standard_type<VectorLikeX>;
    static_assert(hgb_real_type<T>::value, "hala::dot on the GB300 backend: float or double");
    T r = T(0);
    if (N <= 0) return r;
    if (std::is_same<T, double>::value)
        check_hgb(hgb_dot_f64(engine.handle(), N, (double const *)get_standard_data(x), (double const *)get_standard_data(y),
                              (double *)&r, 0), "hala::dot()");
    else
        check_hgb(hgb_dot_f32(engine.handle(), N, (float const *)get_standard_data(x), (float const *)get_standard_data(y),
                              (float *)&r, 0), "hala::dot()");
    return r;
}
template <bool conjugate = true, class VectorLikeX, class VectorLikeY>
auto dot(gpu_engine const &engine, VectorLikeX const &x, VectorLikeY const &y, int incx = 1, int incy = 1, int N = -1) {
    valid::default_size(x, incx, N);
    return dot<conjugate>(engine, N, x, incx, y, incy);
}
template <class VectorLikeX, class VectorLikeY>
auto dotu(gpu_engine const &engine, VectorLikeX const &x, VectorLikeY const &y, int incx = 1, int incy = 1, int N = -1) {
    valid::default_size(x, incx, N);
    return dot<false>(engine, N, x, incx, y, incy);
}

template <typename FS, class VectorLikeX, class VectorLikeY>
void axpy(gpu_engine const &engine, int N, FS alpha, VectorLikeX const &x, int incx, VectorLikeY &&y, int incy) {
    check_types(x, y);
    engine.check_gpu(x, y);
    hgb_detail::unit_stride(incx, "axpy");
    hgb_detail::unit_stride(incy, "axpy");
    using T = get_standard_type<VectorLikeX>;
    static_assert(hgb_real_type<T>::value, "hala::axpy on the GB300 backend: float or double");
    if (N <= 0) return;
    if (std::is_same<T, double>::value)
        check_hgb(hgb_axpy_f64(engine.handle(), N, (double)alpha, (double const *)get_standard_data(x), (double *)get_standard_data(y)),
                  "hala::axpy()");
    else
        check_hgb(hgb_axpy_f32(engine.handle(), N, (float)alpha, (float const *)get_standard_data(x), (float *)get_standard_data(y)),
                  "hala::axpy()");
}
template <typename FP, class VectorLikeX, class VectorLikeY>
void axpy(gpu_engine const &engine, FP alpha, VectorLikeX const &x, VectorLikeY &&y, int incx = 1, int incy = 1, int N = -1) {
    valid::default_size(x, incx, N);
    axpy(engine, N, alpha, x, incx, y, incy);
}

template <typename FS, class VectorLike>
void scal(gpu_engine const &engine, int N, FS alpha, VectorLike &&x, int incx) {
    check_types(x);
    engine.check_gpu(x);
    hgb_detail::unit_stride(incx, "scal");
    using T = get_standard_type<VectorLike>;
    static_assert(hgb_real_type<T>::value, "hala::scal on the GB300 backend: float or double");
    if (N <= 0) return;
    if (std::is_same<T, double>::value)
        check_hgb(hgb_scal_f64(engine.handle(), N, (double)alpha, (double *)get_standard_data(x)), "hala::scal()");
    else
        check_hgb(hgb_scal_f32(engine.handle(), N, (float)alpha, (float *)get_standard_data(x)), "hala::scal()");
}
template <typename FP, class VectorLike>
void scal(gpu_engine const &engine, FP alpha, VectorLike &&x, int incx = 1, int N = -1) {
    valid::default_size(x, incx, N);
    scal(engine, N, alpha, x, incx);
}

/* index of the largest magnitude (zero-based, as the reference returns cublasIxamax - 1); the
 * solvers call it on batch-sized vectors, so the scan runs on the host */
template <class VectorLikeX>
inline int iamax(gpu_engine const &engine, int N, VectorLikeX const &x, int incx) {
    check_types(x);
    engine.check_gpu(x);
    hgb_detail::unit_stride(incx, "iamax");
    if (N <= 0) return -1;
    using T = get_standard_type<VectorLikeX>;
    std::vector<T> h((size_t)N);
    engine.synchronize();
    gpu_copy_n<copy_direction::device2host>(get_standard_data(x), (size_t)N, h.data());
    int best = 0;
    for (int i = 1; i < N; i++)
        if (std::abs(h[i]) > std::abs(h[best])) best = i;
    return best;
}
template <class VectorLikeX>
inline int iamax(gpu_engine const &engine, VectorLikeX const &x, int incx = 1, int N = -1) {
    valid::default_size(x, incx, N);
    return iamax(engine, N, x, incx);
}

/* ------------------------------------------------------- dense tall-skinny BLAS-2 ------ */
/* y = alpha op(A) x + beta y, A column-major M x N with lda == M: the Krylov projection and
 * combination of GMRES (hex/solvers/hala_solvers_gmres.hpp:65-80) and the column sums of the
 * batch reductions (wax/hala_blas_extensions.hpp:246); N <= 64. */
template <typename FPA, typename FPB, class VectorLikeA, class VectorLikeX, class VectorLikeY>
void gemv(gpu_engine const &engine, char trans, int M, int N, FPA alpha, VectorLikeA const &A, int lda,
          VectorLikeX const &x, int incx, FPB beta, VectorLikeY &&y, int incy) {
    check_types(A, x, y);
    engine.check_gpu(A, x, y);
    hgb_detail::unit_stride(incx, "gemv");
    hgb_detail::unit_stride(incy, "gemv");
    if (lda != M) throw std::runtime_error("hala::gemv: the GB300 backend takes lda == M");
    using T = get_standard_type<VectorLikeA>;
    static_assert(hgb_real_type<T>::value, "hala::gemv on the GB300 backend: float or double");
    const bool nt = (trans == 'N' || trans == 'n');
    check_set_size((beta == FPB(0)), y, nt ? M : N);
    if (std::is_same<T, double>::value)
        check_hgb(hgb_gemv_f64(engine.handle(), trans, M, N, (double)alpha, (double const *)get_standard_data(A),
                               (double const *)get_standard_data(x), (double)beta, (double *)get_standard_data(y)),
                  "hala::gemv()");
    else
        check_hgb(hgb_gemv_f32(engine.handle(), trans, M, N, (float)alpha, (float const *)get_standard_data(A),
                               (float const *)get_standard_data(x), (float)beta, (float *)get_standard_data(y)),
                  "hala::gemv()");
}
template <typename FPA, typename FPB, class VectorLikeA, class VectorLikeX, class VectorLikeY>
void gemv(gpu_engine const &engine, char trans, int M, int N, FPA alpha, VectorLikeA const &A, VectorLikeX const &x,
          FPB beta, VectorLikeY &&y, int lda = -1, int incx = 1, int incy = 1) {
    valid::default_ld(M, lda);
    gemv(engine, trans, M, N, alpha, A, lda, x, incx, beta, y, incy);
}

/* C = diag(x) A (side 'L') or A diag(x) (side 'R'), column-major M x N, packed (lda = ldc = M):
 * the column scalings of the batch operations (wax/hala_blas_extensions.hpp:211-265) */
template <class VectorLikeA, class VectorLikeB, class VectorLikeC>
inline void dgmm(gpu_engine const &engine, char side, int M, int N, VectorLikeA const &A, int lda, VectorLikeB const &x,
                 int incx, VectorLikeC &&C, int ldc) {
    check_types(A, x, C);
    engine.check_gpu(A, x, C);
    hgb_detail::unit_stride(incx, "dgmm");
    if (lda != M || ldc != M) throw std::runtime_error("hala::dgmm: the GB300 backend takes packed columns");
    check_set_size(assume_output, C, M, N);
    using T = get_standard_type<VectorLikeA>;
    static_assert(hgb_real_type<T>::value, "hala::dgmm on the GB300 backend: float or double");
    if (std::is_same<T, double>::value)
        check_hgb(hgb_dgmm_f64(engine.handle(), side, M, N, (double const *)get_standard_data(A),
                               (double const *)get_standard_data(x), (double *)get_standard_data(C)), "hala::dgmm()");
    else
        check_hgb(hgb_dgmm_f32(engine.handle(), side, M, N, (float const *)get_standard_data(A),
                               (float const *)get_standard_data(x), (float *)get_standard_data(C)), "hala::dgmm()");
}
template <class VectorLikeA, class VectorLikeB, class VectorLikeC>
inline void dgmm(gpu_engine const &engine, char side, int M, int N, VectorLikeA const &A, VectorLikeB const &x,
                 VectorLikeC &&C, int lda = -1, int incx = 1, int ldc = -1) {
    valid::default_ld(M, lda);
    valid::default_ld(M, ldc);
    dgmm(engine, side, M, N, A, lda, x, incx, C, ldc);
}

/* triangular banded solve, bandwidth 0 only: x_i <- x_i / A_i (unit diag: unchanged), the
 * element-wise division vdivide (wax/hala_blas_extensions.hpp:267-276) builds from it for the
 * per-column scalars of the batch CG; those vectors hold one entry per right-hand side, so the
 * division runs on the host */
template <class VectorLikeA, class VectorLikeX>
inline void tbsv(gpu_engine const &engine, char uplo, char trans, char diag, int N, int k, VectorLikeA const &A, int lda,
                 VectorLikeX &&x, int incx) {
    (void)uplo;
    (void)trans;
    check_types(A, x);
    engine.check_gpu(A, x);
    hgb_detail::unit_stride(incx, "tbsv");
    if (k != 0 || lda != 1) throw std::runtime_error("hala::tbsv: the GB300 backend solves diagonal (k = 0) systems only");
    if (N <= 0 || diag == 'U' || diag == 'u') return;
    using T = get_standard_type<VectorLikeX>;
    std::vector<T> a((size_t)N), h((size_t)N);
    engine.synchronize();
    gpu_copy_n<copy_direction::device2host>(get_standard_data(A), (size_t)N, a.data());
    gpu_copy_n<copy_direction::device2host>(get_standard_data(x), (size_t)N, h.data());
    for (int i = 0; i < N; i++) h[i] /= a[i];
    gpu_copy_n<copy_direction::host2device>(h.data(), (size_t)N, get_standard_data(x));
}
template <class VectorLikeA, class VectorLikeX>
inline void tbsv(gpu_engine const &engine, char uplo, char trans, char diag, int N, int k, VectorLikeA const &A,
                 VectorLikeX &&x, int lda = -1, int incx = 1) {
    valid::default_ld(k + 1, lda);
    tbsv(engine, uplo, trans, diag, N, k, A, lda, x, incx);
}

/* ------------------------------------------------------------------- sparse matrix ----- */
/* gpu_sparse_matrix, gpu/hala_cuda_sparse_general.hpp:192-375: a non-owning view of the device
 * CSR arrays (general.hpp:202) with the kernels' cached analysis; no work buffer is needed, so the
 * buffer sizes are 0 and buffers are accepted and ignored. */
template <typename T>
struct gpu_sparse_matrix {
    using value_type = T;
    static_assert(hgb_real_type<T>::value, "gpu_sparse_matrix on the GB300 backend: float or double");

    template <class VectorLikeP, class VectorLikeI, class VectorLikeV>
    gpu_sparse_matrix(gpu_engine const &engine, int num_rows, int num_cols, int num_nz, VectorLikeP const &pntr,
                      VectorLikeI const &indx, VectorLikeV const &vals)
        : rengine(engine), rows(num_rows), cols(num_cols) {
        hgb_csr *A = nullptr;
        check_hgb(hgb_csr_create(engine.handle(), num_rows, num_cols, num_nz, get_standard_data(pntr), get_standard_data(indx),
                                 (void const *)get_standard_data(vals), hgb_real_type<T>::dtype, &A),
                  "hala::make_sparse_matrix()");
        h = std::shared_ptr<hgb_csr>(A, [](hgb_csr *p) { hgb_csr_destroy(p); });
    }
    template <class VectorLikeP, class VectorLikeI, class VectorLikeV>
    gpu_sparse_matrix(gpu_engine const &engine, int num_cols, VectorLikeP const &pntr, VectorLikeI const &indx,
                      VectorLikeV const &vals)
        : gpu_sparse_matrix(engine, get_size_int(pntr) - 1, num_cols, get_size_int(indx), pntr, indx, vals) {}
    gpu_sparse_matrix(gpu_sparse_matrix const &) = delete;
    gpu_sparse_matrix &operator=(gpu_sparse_matrix const &) = delete;
    gpu_sparse_matrix(gpu_sparse_matrix &&) = default;
    gpu_sparse_matrix &operator=(gpu_sparse_matrix &&) = default;

    template <typename FPa, class VectorLikeX, typename FPb, class VectorLikeY>
    size_t gemv_buffer_size(char, FPa, VectorLikeX const &, FPb, VectorLikeY &&) const { return 0; }
    template <typename FPa, class VectorLikeX, typename FPb, class VectorLikeY, class VectorLikeBuff>
    void gemv(char trans, FPa alpha, VectorLikeX const &x, FPb beta, VectorLikeY &&y, VectorLikeBuff &&) const {
        gemv(trans, alpha, x, beta, y);
    }
    template <typename FPa, class VectorLikeX, typename FPb, class VectorLikeY>
    void gemv(char trans, FPa alpha, VectorLikeX const &x, FPb beta, VectorLikeY &&y) const {
        check_types(x, y);
        rengine.check_gpu(x, y);
        const bool nt = (trans == 'N' || trans == 'n');
        check_set_size((beta == FPb(0)), y, nt ? rows : cols);
        check_hgb(hgb_csr_gemv(h.get(), trans, (double)alpha, (void const *)get_standard_data(x), (double)beta,
                               (void *)get_standard_data(y)), "hala::gpu_sparse_matrix::gemv()");
    }
    /* C = alpha op(A) op(B) + beta C, B dense column-major with b_cols columns (transb 'N') */
    template <typename FSA, class VectorLikeB, typename FSB, class VectorLikeC>
    size_t gemm_buffer_size(char, char, int, int, FSA, VectorLikeB const &, int, FSB, VectorLikeC &, int) const { return 0; }
    template <typename FSA, class VectorLikeB, typename FSB, class VectorLikeC, class VectorLikeT>
    void gemm(char transa, char transb, int b_rows, int b_cols, FSA alpha, VectorLikeB const &B, int ldb, FSB beta,
              VectorLikeC &C, int ldc, VectorLikeT &&) const {
        gemm(transa, transb, b_rows, b_cols, alpha, B, ldb, beta, C, ldc);
    }
    template <typename FSA, class VectorLikeB, typename FSB, class VectorLikeC>
    void gemm(char transa, char transb, int b_rows, int b_cols, FSA alpha, VectorLikeB const &B, int ldb, FSB beta,
              VectorLikeC &C, int ldc) const {
        if (transa != 'N' && transa != 'n') throw std::runtime_error("hala::gpu_sparse_matrix::gemm: transa 'N'");
        if (transb != 'N' && transb != 'n') throw std::runtime_error("hala::gpu_sparse_matrix::gemm: transb 'N'");
        (void)b_rows;
        check_set_size((beta == FSB(0)), C, hala_size(ldc, b_cols));
        check_hgb(hgb_csr_gemm(h.get(), b_cols, (double)alpha, (void const *)get_standard_data(B), ldb, (double)beta,
                               (void *)get_standard_data(C), ldc), "hala::gpu_sparse_matrix::gemm()");
    }
    gpu_engine const &engine() const { return rengine; }
    hgb_csr *handle() const { return h.get(); }

private:
    gpu_engine rengine;
    int rows, cols;
    std::shared_ptr<hgb_csr> h;
};

template <class VectorLikeP, class VectorLikeI, class VectorLikeV>
auto make_sparse_matrix(gpu_engine const &engine, int num_rows, int num_cols, int num_nz, VectorLikeP const &pntr,
                        VectorLikeI const &indx, VectorLikeV const &vals) {
    return gpu_sparse_matrix<get_standard_type<VectorLikeV>>(engine, num_rows, num_cols, num_nz, pntr, indx, vals);
}
template <class VectorLikeP, class VectorLikeI, class VectorLikeV>
auto make_sparse_matrix(gpu_engine const &engine, int num_cols, VectorLikeP const &pntr, VectorLikeI const &indx,
                        VectorLikeV const &vals) {
    return gpu_sparse_matrix<get_standard_type<VectorLikeV>>(engine, num_cols, pntr, indx, vals);
}

/* sparse_gemv(gpu_engine, trans, M, N, alpha, pntr, indx, vals, x, beta, y), general.hpp:407-419 */
template <typename FPa, class VectorLikeP, class VectorLikeI, class VectorLikeV, class VectorLikeX, typename FPb, class VectorLikeY>
void sparse_gemv(gpu_engine const &engine, char trans, int M, int N, FPa alpha, VectorLikeP const &pntr,
                 VectorLikeI const &indx, VectorLikeV const &vals, VectorLikeX const &x, FPb beta, VectorLikeY &&y) {
    auto matrix = make_sparse_matrix(engine, M, N, get_size_int(indx), pntr, indx, vals);
    matrix.gemv(trans, alpha, x, beta, y);
}
/* sparse_gemm(gpu_engine, ...), general.hpp:425-441 */
template <typename FSA, class VectorLikeP, class VectorLikeI, class VectorLikeV, class VectorLikeB, typename FSB, class VectorLikeC>
void sparse_gemm(gpu_engine const &engine, char transa, char transb, int M, int N, int K, FSA alpha, VectorLikeP const &pntr,
                 VectorLikeI const &indx, VectorLikeV const &vals, VectorLikeB const &B, int ldb, FSB beta, VectorLikeC &&C,
                 int ldc) {
    auto matrix = make_sparse_matrix(engine, M, K, get_size_int(indx), pntr, indx, vals);
    matrix.gemm(transa, transb, K, N, alpha, B, ldb, beta, C, ldc);
}

/* ------------------------------------------------------------------ triangular --------- */
/* gpu_triangular_matrix, gpu/hala_cuda_sparse_triangular.hpp:38-421: the triangle (uplo) of a
 * CSR matrix that may hold both (the reference's fill mode), unit or non-unit diagonal */
template <typename T>
struct gpu_triangular_matrix {
    using value_type = T;
    template <class VectorLikeP, class VectorLikeI, class VectorLikeV>
    gpu_triangular_matrix(gpu_engine const &engine, char uplo, char diag, VectorLikeP const &pntr, VectorLikeI const &indx,
                          VectorLikeV const &vals, char = 'L')
        : rengine(engine), rows(get_size_int(pntr) - 1) {
        hgb_tri *t = nullptr;
        check_hgb(hgb_tri_create(engine.handle(), uplo, diag, rows, get_size_int(indx), get_standard_data(pntr),
                                 get_standard_data(indx), (void const *)get_standard_data(vals), hgb_real_type<T>::dtype, &t),
                  "hala::make_triangular_matrix()");
        h = std::shared_ptr<hgb_tri>(t, [](hgb_tri *p) { hgb_tri_destroy(p); });
    }
    gpu_triangular_matrix(gpu_triangular_matrix const &) = delete;
    gpu_triangular_matrix(gpu_triangular_matrix &&) = default;
    template <typename FPA, class VectorLikeB, class VectorLikeX>
    size_t trsv_buffer_size(char, FPA, VectorLikeB const &, VectorLikeX &&) const { return 0; }
    template <typename FPA, class VectorLikeB, class VectorLikeX, class VectorLikeT>
    void trsv(char trans, FPA alpha, VectorLikeB const &b, VectorLikeX &&x, VectorLikeT &&) const { trsv(trans, alpha, b, x); }
    template <typename FPA, class VectorLikeB, class VectorLikeX>
    void trsv(char trans, FPA alpha, VectorLikeB const &b, VectorLikeX &&x) const {
        check_types(b, x);
        check_set_size(assume_output, x, rows);
        check_hgb(hgb_tri_solve(h.get(), trans, (double)alpha, (void const *)get_standard_data(b), (void *)get_standard_data(x)),
                  "hala::gpu_triangular_matrix::trsv()");
    }
    /* B <- op(T)^-1 alpha B, column by column (nrhs columns of leading dimension ldb) */
    template <typename FPA, class VectorLikeB>
    size_t trsm_buffer_size(char, char, int, FPA, VectorLikeB const &, int = -1) const { return 0; }
    template <typename FPA, class VectorLikeB, class VectorLikeT>
    void trsm(char transa, char transb, int nrhs, FPA alpha, VectorLikeB &&B, int ldb, VectorLikeT &&) const {
        trsm(transa, transb, nrhs, alpha, B, ldb);
    }
    template <typename FPA, class VectorLikeB>
    void trsm(char transa, char transb, int nrhs, FPA alpha, VectorLikeB &&B, int ldb = -1) const {
        if (transb != 'N' && transb != 'n') throw std::runtime_error("hala::gpu_triangular_matrix::trsm: transb 'N'");
        if (ldb < 0) ldb = rows;
        gpu_vector<T> col((size_t)rows, rengine.device());
        T *base = get_standard_data(B);
        for (int c = 0; c < nrhs; c++) {
            gpu_copy_n<copy_direction::device2device>(base + (size_t)c * ldb, (size_t)rows, col.data());
            check_hgb(hgb_tri_solve(h.get(), transa, (double)alpha, col.data(), base + (size_t)c * ldb),
                      "hala::gpu_triangular_matrix::trsm()");
        }
    }
    gpu_engine const &engine() const { return rengine; }

private:
    gpu_engine rengine;
    int rows;
    std::shared_ptr<hgb_tri> h;
};

template <class VectorLikeP, class VectorLikeI, class VectorLikeV>
auto make_triangular_matrix(gpu_engine const &engine, char uplo, char diag, VectorLikeP const &pntr,
                            VectorLikeI const &indx, VectorLikeV const &vals, char policy = 'L') {
    return gpu_triangular_matrix<get_standard_type<VectorLikeV>>(engine, uplo, diag, pntr, indx, vals, policy);
}

/* --------------------------------------------------------------------------- ILU ------- */
/* gpu_ilu, gpu/hala_gpu_ilu.hpp:45-185: owns its copy of the factor (gpu_ilu.hpp:64), aliases the
 * pattern; the factor and the sweeps have the reference's CPU arithmetic (factorize_ilu_array,
 * apply_ilu_array, sparse/hala_sparse_utils.hpp:229-276), bit for bit. */
template <typename T>
struct gpu_ilu {
    using value_type = T;
    using engine_type = gpu_engine;
    static_assert(hgb_real_type<T>::value, "gpu_ilu on the GB300 backend: float or double");

    template <class VectorLikeP, class VectorLikeI, class VectorLikeV>
    gpu_ilu(gpu_engine const &cengine, VectorLikeP const &mpntr, VectorLikeI const &mindx, VectorLikeV const &mvals, char policy)
        : rengine(cengine), num_rows(get_size_int(mpntr) - 1) {
        hgb_ilu *M = nullptr;
        const int st = hgb_ilu0_create(cengine.handle(), num_rows, get_size_int(mindx), get_standard_data(mpntr),
                                       get_standard_data(mindx), (void const *)get_standard_data(mvals),
                                       hgb_real_type<T>::dtype, hgb_real_type<T>::dtype, policy, &M);
        if (st != HGB_OK && st != HGB_ERR_ZERO_PIVOT) check_hgb(st, "hala::make_ilu()");
        h = std::shared_ptr<hgb_ilu>(M, [](hgb_ilu *p) { hgb_ilu0_destroy(p); });
    }
    gpu_ilu(gpu_ilu const &) = delete;
    gpu_ilu &operator=(gpu_ilu const &) = delete;
    gpu_ilu(gpu_ilu &&) = default;
    gpu_ilu &operator=(gpu_ilu &&) = default;

    template <class VectorLikeX, class VectorLikeR>
    size_t buffer_size(VectorLikeX const &, VectorLikeR &&, int) const { return 0; }
    template <class VectorLikeX, class VectorLikeR>
    gpu_vector<value_type> get_temp_buffer(VectorLikeX const &, VectorLikeR &&, int) const {
        return gpu_vector<value_type>(rengine.device());
    }
    /* r = U^-1 L^-1 x for num_rhs column-major right-hand sides */
    template <class VectorLikeX, class VectorLikeR, class VectorLikeT>
    void apply(VectorLikeX const &x, VectorLikeR &&r, int num_rhs, VectorLikeT &&) const {
        apply(x, r, num_rhs);
    }
    template <class VectorLikeX, class VectorLikeR>
    void apply(VectorLikeX const &x, VectorLikeR &&r, int num_rhs = 1) const {
        check_types(x, r);
        check_set_size(assume_output, r, num_rhs, num_rows);
        if (num_rhs == 1)
            check_hgb(hgb_ilu0_apply(h.get(), 'N', (void const *)get_standard_data(x), (void *)get_standard_data(r)),
                      "hala::gpu_ilu::apply()");
        else
            check_hgb(hgb_ilu0_apply_nrhs(h.get(), 'N', num_rhs, (void const *)get_standard_data(x),
                                          (void *)get_standard_data(r)), "hala::gpu_ilu::apply()");
    }
    gpu_engine const &engine() const { return rengine; }
    hgb_ilu *handle() const { return h.get(); }

private:
    gpu_engine rengine;
    int num_rows;
    std::shared_ptr<hgb_ilu> h;
};

template <class VectorLikeP, class VectorLikeI, class VectorLikeV>
auto make_ilu(gpu_engine const &cengine, VectorLikeP const &pntr, VectorLikeI const &indx, VectorLikeV const &vals,
              char policy = 'N') {
    return gpu_ilu<get_standard_type<VectorLikeV>>(cengine, pntr, indx, vals, policy);
}

}  // namespace hala

#endif
