// Anisotropic field update (materials/tensor.py:437-590 AnisotropicUpdater):
//   E' = E + (dt/eps0) [eps]^-1 curl H,   H' = H - (dt/mu0) [mu]^-1 curl E
// elementwise over arrays of the same shape.  Diagonal tensors divide by the
// diagonal (tensor.py:508-512, 561-565), full tensors multiply by the inverse
// (tensor.py:513-535, 566-588); the coefficients are per cell or uniform.  Every
// operation is rounded explicitly, in the order the reference's array expressions
// evaluate, so that float64 results equal NumPy's bit for bit.
#include "pc_internal.cuh"

namespace pc {
namespace {

template <typename T>
struct Ops;
template <>
struct Ops<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};
template <>
struct Ops<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};

struct AnisoArgs {
    const void* f[3];
    const void* curl[3];
    void* out[3];
    const void* coef;   // per cell: [k][n] (k = 3 diagonal, 9 full, row-major), or null
    double cu[9];       // uniform coefficients when coef is null
    double scale;       // dt / eps0 or dt / mu0
    int64_t n;
    int sign;           // +1: E update, -1: H update
};

template <typename T, bool DIAG>
__global__ void __launch_bounds__(256) aniso_update(AnisoArgs a) {
    using O = Ops<T>;
    const T* f0 = static_cast<const T*>(a.f[0]);
    const T* f1 = static_cast<const T*>(a.f[1]);
    const T* f2 = static_cast<const T*>(a.f[2]);
    const T* c0 = static_cast<const T*>(a.curl[0]);
    const T* c1 = static_cast<const T*>(a.curl[1]);
    const T* c2 = static_cast<const T*>(a.curl[2]);
    T* o[3] = {static_cast<T*>(a.out[0]), static_cast<T*>(a.out[1]), static_cast<T*>(a.out[2])};
    const T* cf = static_cast<const T*>(a.coef);
    const T s = (T)a.scale;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        const T f[3] = {f0[i], f1[i], f2[i]};
        const T c[3] = {c0[i], c1[i], c2[i]};
        auto k = [&](int q) { return cf ? cf[(int64_t)q * a.n + i] : (T)a.cu[q]; };
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            T v;
            if (DIAG) {
                // E + s * c / d   or   H - s * c / d
                const T d = O::div(O::mul(s, c[r]), k(r));
                v = a.sign > 0 ? O::add(f[r], d) : O::sub(f[r], d);
            } else {
                // d = +-s * ((m0 c0 + m1 c1) + m2 c2); F + d
                const T m = O::add(O::add(O::mul(k(3 * r), c[0]), O::mul(k(3 * r + 1), c[1])), O::mul(k(3 * r + 2), c[2]));
                const T d = O::mul(a.sign > 0 ? s : -s, m);
                v = O::add(f[r], d);
            }
            o[r][i] = v;
        }
    }
}

}  // namespace
}  // namespace pc

using namespace pc;

int pc_aniso_update(int32_t precision, int32_t diagonal, int32_t sign, const void* const fields[3],
                    const void* const curls[3], void* const out[3], int64_t n, const void* d_coef,
                    const double* coef_uniform, double scale, void* stream) {
    if ((precision != 4 && precision != 8) || n < 0 || !fields || !curls || !out || (sign != 1 && sign != -1))
        return PC_ERR_INVALID;
    if (!d_coef && !coef_uniform) return PC_ERR_INVALID;
    if (n == 0) return PC_OK;
    AnisoArgs a{};
    for (int q = 0; q < 3; ++q) {
        if (!fields[q] || !curls[q] || !out[q]) return PC_ERR_INVALID;
        a.f[q] = fields[q];
        a.curl[q] = curls[q];
        a.out[q] = out[q];
    }
    a.coef = d_coef;
    if (!d_coef)
        for (int q = 0; q < (diagonal ? 3 : 9); ++q) a.cu[q] = coef_uniform[q];
    a.scale = scale;
    a.n = n;
    a.sign = sign;
    cudaStream_t s = (cudaStream_t)stream;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
    if (precision == 8) {
        if (diagonal)
            aniso_update<double, true><<<blocks, 256, 0, s>>>(a);
        else
            aniso_update<double, false><<<blocks, 256, 0, s>>>(a);
    } else {
        if (diagonal)
            aniso_update<float, true><<<blocks, 256, 0, s>>>(a);
        else
            aniso_update<float, false><<<blocks, 256, 0, s>>>(a);
    }
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}
