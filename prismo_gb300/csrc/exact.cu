// Kernels whose float64 results must equal the reference NumPy arithmetic bit for
// bit.  This translation unit is compiled with -fmad=false so that no a*b+c is
// contracted into an FMA, and every quotient is a true IEEE division, matching
// NumPy's evaluation order term by term.
//
//   * coefficient build      core/solver.py:113-133 (Ca, Cb, Da, Db per cell)
//                            core/solver.py:458-533 (interpolation to Yee points)
//   * reference stepper      core/solver.py:167-456 (PC_MODE_LEGACY)
//   * soft sources           sources/point.py:47-73, sources/plane_wave.py:184-221
#include "pc_internal.cuh"

namespace pc {

namespace {

__device__ __forceinline__ void cell_e(const double* eps, const double* sig, int64_t c, double dt,
                                       double eps0, double& ca, double& cb) {
    const double er = eps ? eps[c] : 1.0;
    const double e = eps0 * er;
    if (!sig) {  // sigma = 0: q = 0, so Ca = 1 / 1 and Cb = (dt / e) / 1 exactly
        ca = 1.0;
        cb = dt / e;
        return;
    }
    const double s = sig[c];
    const double q = s * dt / (2.0 * e);
    ca = (1.0 - q) / (1.0 + q);
    cb = (dt / e) / (1.0 + q);
}

__device__ __forceinline__ void cell_h(const double* mu, const double* sigm, int64_t c, double dt,
                                       double mu0, double& da, double& db) {
    const double mr = mu ? mu[c] : 1.0;
    const double s = sigm ? sigm[c] : 0.0;
    const double m = mu0 * mr;
    const double q = s * dt / (2.0 * m);
    da = (1.0 - q) / (1.0 + q);
    db = (dt / m) / (1.0 + q);
}

struct CoefOut {
    void* ca[3];
    void* cb[3];
    void* da[3];
    void* db[3];
};

template <typename T>
__device__ __forceinline__ void put(void* p, int64_t o, double v) {
    if (p) reinterpret_cast<T*>(p)[o] = static_cast<T>(v);
}

// One thread per padded position (i, j, k < pitch).
template <typename T>
__global__ void build_coef3(int nx, int ny, int nz, int pitch, const double* eps, const double* mu,
                            const double* sig, const double* sigm, double dt, double eps0, double mu0,
                            CoefOut out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= pitch || j >= ny || i >= nx) return;
    const int64_t o = ((int64_t)i * ny + j) * pitch + k;
    auto cid = [&](int ii, int jj, int kk) { return ((int64_t)ii * ny + jj) * nz + kk; };
    double a0, b0, a1, b1, a2, b2, a3, b3;
    // Ex: (i, j+1/2, k+1/2), 4-point mean over y and z
    if (j < ny - 1 && k < nz - 1) {
        cell_e(eps, sig, cid(i, j, k), dt, eps0, a0, b0);
        cell_e(eps, sig, cid(i, j + 1, k), dt, eps0, a1, b1);
        cell_e(eps, sig, cid(i, j, k + 1), dt, eps0, a2, b2);
        cell_e(eps, sig, cid(i, j + 1, k + 1), dt, eps0, a3, b3);
        put<T>(out.ca[0], o, 0.25 * (a0 + a1 + a2 + a3));
        put<T>(out.cb[0], o, 0.25 * (b0 + b1 + b2 + b3));
    } else {
        put<T>(out.ca[0], o, 0.0);
        put<T>(out.cb[0], o, 0.0);
    }
    // Ey: (i+1/2, j, k+1/2), mean over x and z
    if (i < nx - 1 && k < nz - 1) {
        cell_e(eps, sig, cid(i, j, k), dt, eps0, a0, b0);
        cell_e(eps, sig, cid(i + 1, j, k), dt, eps0, a1, b1);
        cell_e(eps, sig, cid(i, j, k + 1), dt, eps0, a2, b2);
        cell_e(eps, sig, cid(i + 1, j, k + 1), dt, eps0, a3, b3);
        put<T>(out.ca[1], o, 0.25 * (a0 + a1 + a2 + a3));
        put<T>(out.cb[1], o, 0.25 * (b0 + b1 + b2 + b3));
    } else {
        put<T>(out.ca[1], o, 0.0);
        put<T>(out.cb[1], o, 0.0);
    }
    // Ez: (i+1/2, j+1/2, k), mean over x and y
    if (i < nx - 1 && j < ny - 1 && k < nz) {
        cell_e(eps, sig, cid(i, j, k), dt, eps0, a0, b0);
        cell_e(eps, sig, cid(i + 1, j, k), dt, eps0, a1, b1);
        cell_e(eps, sig, cid(i, j + 1, k), dt, eps0, a2, b2);
        cell_e(eps, sig, cid(i + 1, j + 1, k), dt, eps0, a3, b3);
        put<T>(out.ca[2], o, 0.25 * (a0 + a1 + a2 + a3));
        put<T>(out.cb[2], o, 0.25 * (b0 + b1 + b2 + b3));
    } else {
        put<T>(out.ca[2], o, 0.0);
        put<T>(out.cb[2], o, 0.0);
    }
    if (!out.da[0] && !out.db[0] && !out.da[1] && !out.db[1] && !out.da[2] && !out.db[2]) return;
    // Hx: (i+1/2, j, k), mean over x
    if (i < nx - 1 && k < nz) {
        cell_h(mu, sigm, cid(i, j, k), dt, mu0, a0, b0);
        cell_h(mu, sigm, cid(i + 1, j, k), dt, mu0, a1, b1);
        put<T>(out.da[0], o, 0.5 * (a0 + a1));
        put<T>(out.db[0], o, 0.5 * (b0 + b1));
    } else {
        put<T>(out.da[0], o, 0.0);
        put<T>(out.db[0], o, 0.0);
    }
    // Hy: (i, j+1/2, k), mean over y
    if (j < ny - 1 && k < nz) {
        cell_h(mu, sigm, cid(i, j, k), dt, mu0, a0, b0);
        cell_h(mu, sigm, cid(i, j + 1, k), dt, mu0, a1, b1);
        put<T>(out.da[1], o, 0.5 * (a0 + a1));
        put<T>(out.db[1], o, 0.5 * (b0 + b1));
    } else {
        put<T>(out.da[1], o, 0.0);
        put<T>(out.db[1], o, 0.0);
    }
    // Hz: (i, j, k+1/2), mean over z
    if (k < nz - 1) {
        cell_h(mu, sigm, cid(i, j, k), dt, mu0, a0, b0);
        cell_h(mu, sigm, cid(i, j, k + 1), dt, mu0, a1, b1);
        put<T>(out.da[2], o, 0.5 * (a0 + a1));
        put<T>(out.db[2], o, 0.5 * (b0 + b1));
    } else {
        put<T>(out.da[2], o, 0.0);
        put<T>(out.db[2], o, 0.0);
    }
}

// 2D: cells (i, j, 0) of (nx, ny, 1) material arrays; padded layout i*pitch + j.
template <typename T>
__global__ void build_coef2(int nx, int ny, int pitch, const double* eps, const double* mu,
                            const double* sig, const double* sigm, double dt, double eps0, double mu0,
                            CoefOut out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= pitch || i >= nx) return;
    const int64_t o = (int64_t)i * pitch + j;
    auto cid = [&](int ii, int jj) { return (int64_t)ii * ny + jj; };
    double a0, b0, a1, b1, a2, b2, a3, b3;
    if (j < ny - 1) {  // Ex (i, j+1/2): mean over y
        cell_e(eps, sig, cid(i, j), dt, eps0, a0, b0);
        cell_e(eps, sig, cid(i, j + 1), dt, eps0, a1, b1);
        put<T>(out.ca[0], o, 0.5 * (a0 + a1));
        put<T>(out.cb[0], o, 0.5 * (b0 + b1));
    } else {
        put<T>(out.ca[0], o, 0.0);
        put<T>(out.cb[0], o, 0.0);
    }
    if (i < nx - 1 && j < ny) {  // Ey (i+1/2, j): mean over x
        cell_e(eps, sig, cid(i, j), dt, eps0, a0, b0);
        cell_e(eps, sig, cid(i + 1, j), dt, eps0, a1, b1);
        put<T>(out.ca[1], o, 0.5 * (a0 + a1));
        put<T>(out.cb[1], o, 0.5 * (b0 + b1));
    } else {
        put<T>(out.ca[1], o, 0.0);
        put<T>(out.cb[1], o, 0.0);
    }
    if (i < nx - 1 && j < ny - 1) {  // Ez (i+1/2, j+1/2): 4-point mean
        cell_e(eps, sig, cid(i, j), dt, eps0, a0, b0);
        cell_e(eps, sig, cid(i + 1, j), dt, eps0, a1, b1);
        cell_e(eps, sig, cid(i, j + 1), dt, eps0, a2, b2);
        cell_e(eps, sig, cid(i + 1, j + 1), dt, eps0, a3, b3);
        put<T>(out.ca[2], o, 0.25 * (a0 + a1 + a2 + a3));
        put<T>(out.cb[2], o, 0.25 * (b0 + b1 + b2 + b3));
    } else {
        put<T>(out.ca[2], o, 0.0);
        put<T>(out.cb[2], o, 0.0);
    }
    if (i < nx - 1 && j < ny) {  // Hx (i+1/2, j): mean over x
        cell_h(mu, sigm, cid(i, j), dt, mu0, a0, b0);
        cell_h(mu, sigm, cid(i + 1, j), dt, mu0, a1, b1);
        put<T>(out.da[0], o, 0.5 * (a0 + a1));
        put<T>(out.db[0], o, 0.5 * (b0 + b1));
    } else {
        put<T>(out.da[0], o, 0.0);
        put<T>(out.db[0], o, 0.0);
    }
    if (j < ny - 1) {  // Hy (i, j+1/2): mean over y
        cell_h(mu, sigm, cid(i, j), dt, mu0, a0, b0);
        cell_h(mu, sigm, cid(i, j + 1), dt, mu0, a1, b1);
        put<T>(out.da[1], o, 0.5 * (a0 + a1));
        put<T>(out.db[1], o, 0.5 * (b0 + b1));
    } else {
        put<T>(out.da[1], o, 0.0);
        put<T>(out.db[1], o, 0.0);
    }
    if (j < ny) {  // Hz (i, j): the cell value itself
        cell_h(mu, sigm, cid(i, j), dt, mu0, a0, b0);
        put<T>(out.da[2], o, a0);
        put<T>(out.db[2], o, b0);
    } else {
        put<T>(out.da[2], o, 0.0);
        put<T>(out.db[2], o, 0.0);
    }
}

// ---------------------------------------------------------------------------
// Reference stepper (PC_MODE_LEGACY), in place: H from E, then E from H.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T coef(const T* p, int64_t o, T s) {
    return p ? p[o] : s;
}

// core/solver.py:167-253: forward differences written into H[:, :-2, :-2]-style slices.
template <typename T>
__global__ void legacy_h3(FieldArgs<T> a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (k >= nz || j >= ny) return;
    const int64_t P = a.pitch, R = (int64_t)ny * P;
    const int64_t o = ((int64_t)i * ny + j) * P + k;
    const T *Ex = a.Ein[0], *Ey = a.Ein[1], *Ez = a.Ein[2];
    T *Hx = a.Hout[0], *Hy = a.Hout[1], *Hz = a.Hout[2];
    if (i < nx - 1 && j < ny - 2 && k < nz - 2) {
        const T cy = (Ez[o + P] - Ez[o]) / a.dy;
        const T cz = (Ey[o + 1] - Ey[o]) / a.dz;
        Hx[o] = coef(a.da[0], o, a.da_s) * Hx[o] - coef(a.db[0], o, a.db_s) * (cy - cz);
    }
    if (i < nx - 2 && j < ny - 1 && k < nz - 2) {
        const T cz = (Ex[o + 1] - Ex[o]) / a.dz;
        const T cx = (Ez[o + R] - Ez[o]) / a.dx;
        Hy[o] = coef(a.da[1], o, a.da_s) * Hy[o] - coef(a.db[1], o, a.db_s) * (cz - cx);
    }
    if (i < nx - 2 && j < ny - 2 && k < nz - 1) {
        const T cx = (Ey[o + R] - Ey[o]) / a.dx;
        const T cy = (Ex[o + P] - Ex[o]) / a.dy;
        Hz[o] = coef(a.da[2], o, a.da_s) * Hz[o] - coef(a.db[2], o, a.db_s) * (cx - cy);
    }
}

// core/solver.py:255-309 (identical in the corrected stepper without CPML).
template <typename T>
__global__ void legacy_e3(FieldArgs<T> a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (k >= nz || j >= ny) return;
    const int64_t P = a.pitch, R = (int64_t)ny * P;
    const int64_t o = ((int64_t)i * ny + j) * P + k;
    const T *Hx = a.Hin[0], *Hy = a.Hin[1], *Hz = a.Hin[2];
    T *Ex = a.Eout[0], *Ey = a.Eout[1], *Ez = a.Eout[2];
    if (j < ny - 1 && k < nz - 1) {
        const T c1 = (Hz[o + P] - Hz[o]) / a.dy;
        const T c2 = (Hy[o + 1] - Hy[o]) / a.dz;
        Ex[o] = coef(a.ca[0], o, T(1)) * Ex[o] + a.cb[0][o] * (c1 - c2);
    }
    if (i < nx - 1 && k < nz - 1) {
        const T c1 = (Hx[o + 1] - Hx[o]) / a.dz;
        const T c2 = (Hz[o + R] - Hz[o]) / a.dx;
        Ey[o] = coef(a.ca[1], o, T(1)) * Ey[o] + a.cb[1][o] * (c1 - c2);
    }
    if (i < nx - 1 && j < ny - 1) {
        const T c1 = (Hy[o + R] - Hy[o]) / a.dx;
        const T c2 = (Hx[o + P] - Hx[o]) / a.dy;
        Ez[o] = coef(a.ca[2], o, T(1)) * Ez[o] + a.cb[2][o] * (c1 - c2);
    }
}

// np.max(np.abs(F)) > 0 for Ex, Ey, Ez (core/solver.py:321, 367).  Bits per
// component c: 1<<(2c) "some |x| > 0", 1<<(2c+1) "some NaN" (max is then NaN).
template <typename T>
__global__ void legacy_flags2(const T* Ex, const T* Ey, const T* Ez, int nx, int ny, int pitch,
                              uint32_t* flags) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    uint32_t f = 0;
    if (i < nx && j < ny) {
        const int64_t o = (int64_t)i * pitch + j;
        const T v[3] = {Ex[o], Ey[o], Ez[o]};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (v[c] != v[c]) f |= 2u << (2 * c);
            else if (v[c] != T(0)) f |= 1u << (2 * c);
        }
    }
    // warp-aggregate before the atomic
    for (int s = 16; s > 0; s >>= 1) f |= __shfl_xor_sync(0xffffffffu, f, s);
    if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

__device__ __forceinline__ bool fam_on(uint32_t f, int c) {
    return ((f >> (2 * c)) & 3u) == 1u;
}

// core/solver.py:311-397: sign-flipped Ez family into [:, :-2], Hz family with
// zero-padded curls over the whole array; each family skipped when its E is 0.
template <typename T>
__global__ void legacy_h2(FieldArgs<T> a, const uint32_t* flags) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int nx = a.nx, ny = a.ny;
    if (i >= nx || j >= ny) return;
    const uint32_t f = *flags;
    const int64_t P = a.pitch;
    const int64_t o = (int64_t)i * P + j;
    const T *Ex = a.Ein[0], *Ey = a.Ein[1], *Ez = a.Ein[2];
    T *Hx = a.Hout[0], *Hy = a.Hout[1], *Hz = a.Hout[2];
    if (fam_on(f, 2)) {
        if (i < nx - 1 && j < ny - 2) {
            const T cy = (Ez[o + 1] - Ez[o]) / a.dy;
            Hx[o] = coef(a.da[0], o, a.da_s) * Hx[o] + coef(a.db[0], o, a.db_s) * cy;
        }
        if (i < nx - 2 && j < ny - 1) {
            const T cx = (Ez[o + P] - Ez[o]) / a.dx;
            Hy[o] = coef(a.da[1], o, a.da_s) * Hy[o] - coef(a.db[1], o, a.db_s) * cx;
        }
    }
    if (fam_on(f, 0) || fam_on(f, 1)) {
        const T cx = (i < nx - 2) ? (Ey[o + P] - Ey[o]) / a.dx : T(0);
        const T cy = (j < ny - 2) ? (Ex[o + 1] - Ex[o]) / a.dy : T(0);
        Hz[o] = coef(a.da[2], o, a.da_s) * Hz[o] - coef(a.db[2], o, a.db_s) * (cx - cy);
    }
}

// core/solver.py:399-456.
template <typename T>
__global__ void legacy_e2(FieldArgs<T> a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int nx = a.nx, ny = a.ny;
    if (i >= nx || j >= ny) return;
    const int64_t P = a.pitch;
    const int64_t o = (int64_t)i * P + j;
    const T *Hx = a.Hin[0], *Hy = a.Hin[1], *Hz = a.Hin[2];
    T *Ex = a.Eout[0], *Ey = a.Eout[1], *Ez = a.Eout[2];
    if (i < nx - 1 && j < ny - 1) {
        const T c1 = (Hy[o + P] - Hy[o]) / a.dx;
        const T c2 = (Hx[o + 1] - Hx[o]) / a.dy;
        Ez[o] = coef(a.ca[2], o, T(1)) * Ez[o] + a.cb[2][o] * (c1 - c2);
    }
    if (j < ny - 1) {
        const T c = (Hz[o + 1] - Hz[o]) / a.dy;
        Ex[o] = coef(a.ca[0], o, T(1)) * Ex[o] + a.cb[0][o] * c;
    }
    if (i < nx - 1) {
        const T c = (Hz[o + P] - Hz[o]) / a.dx;
        Ey[o] = coef(a.ca[1], o, T(1)) * Ey[o] - a.cb[1][o] * c;
    }
}

// Soft sources: field[off[n]] += w[n] * amp.  One block row per source.
struct SrcLaunch {
    int nsrc;
    int comp[32];
    int n[32];
    const int64_t* off[32];
    const double* w[32];
};

template <typename T>
__global__ void add_sources(SrcLaunch s, T* F0, T* F1, T* F2, T* F3, T* F4, T* F5, const double* amps,
                            int row_stride, int col0) {
    const int si = blockIdx.y;
    if (si >= s.nsrc) return;
    T* F[6] = {F0, F1, F2, F3, F4, F5};
    T* f = F[s.comp[si]];
    const double amp = amps[col0 + si];
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < s.n[si]; n += gridDim.x * blockDim.x) {
        const int64_t o = s.off[si][n];
        const double w = s.w[si][n];
        f[o] = f[o] + static_cast<T>(w * amp);
    }
    (void)row_stride;
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int launch_build_coefficients(const pc_grid_desc& g, const double* eps, const double* mu,
                              const double* sig, const double* sigm, double eps0, double mu0,
                              void* const ca[3], void* const cb[3], void* const da[3],
                              void* const db[3], cudaStream_t s, int64_t* launches) {
    CoefOut out;
    for (int c = 0; c < 3; ++c) {
        out.ca[c] = ca ? ca[c] : nullptr;
        out.cb[c] = cb ? cb[c] : nullptr;
        out.da[c] = da ? da[c] : nullptr;
        out.db[c] = db ? db[c] : nullptr;
    }
    if (g.ndim == 3) {
        dim3 blk(32, 8);
        dim3 grd((g.pitch + 31) / 32, (g.ny + 7) / 8, g.nx);
        if (g.precision == 8)
            build_coef3<double><<<grd, blk, 0, s>>>(g.nx, g.ny, g.nz, g.pitch, eps, mu, sig, sigm, g.dt, eps0,
                                                    mu0, out);
        else
            build_coef3<float><<<grd, blk, 0, s>>>(g.nx, g.ny, g.nz, g.pitch, eps, mu, sig, sigm, g.dt, eps0,
                                                   mu0, out);
    } else {
        dim3 blk(32, 8);
        dim3 grd((g.pitch + 31) / 32, (g.nx + 7) / 8);
        if (g.precision == 8)
            build_coef2<double><<<grd, blk, 0, s>>>(g.nx, g.ny, g.pitch, eps, mu, sig, sigm, g.dt, eps0, mu0, out);
        else
            build_coef2<float><<<grd, blk, 0, s>>>(g.nx, g.ny, g.pitch, eps, mu, sig, sigm, g.dt, eps0, mu0, out);
    }
    ++*launches;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

template <typename T>
static FieldArgs<T> inplace_args(pc_ctx* c) {
    FieldArgs<T> a{};
    const pc_grid_desc& g = c->g;
    a.nx = g.nx;
    a.ny = g.ny;
    a.nz = g.nz;
    a.pitch = g.pitch;
    a.dx = T(g.dx);
    a.dy = T(g.dy);
    a.dz = T(g.dz);
    a.inv_dx = T(1.0 / g.dx);
    a.inv_dy = T(1.0 / g.dy);
    a.inv_dz = g.ndim == 3 ? T(1.0 / g.dz) : T(0);
    for (int q = 0; q < 3; ++q) {
        a.Ein[q] = static_cast<const T*>(c->F[c->cur][q]);
        a.Hin[q] = static_cast<const T*>(c->F[c->cur][3 + q]);
        a.Eout[q] = static_cast<T*>(c->F[c->cur][q]);
        a.Hout[q] = static_cast<T*>(c->F[c->cur][3 + q]);
        a.ca[q] = static_cast<const T*>(c->ca[q]);
        a.cb[q] = static_cast<const T*>(c->cb[q]);
        a.da[q] = static_cast<const T*>(c->da[q]);
        a.db[q] = static_cast<const T*>(c->db[q]);
    }
    a.da_s = T(c->da_s);
    a.db_s = T(c->db_s);
    a.status = c->d_status;
    return a;
}

template <typename T>
static int legacy_step_t(pc_ctx* c, cudaStream_t s) {
    FieldArgs<T> a = inplace_args<T>(c);
    const pc_grid_desc& g = c->g;
    if (g.ndim == 3) {
        dim3 blk(32, 8);
        dim3 grd((g.nz + 31) / 32, (g.ny + 7) / 8, g.nx);
        legacy_h3<T><<<grd, blk, 0, s>>>(a);
        legacy_e3<T><<<grd, blk, 0, s>>>(a);
        c->launches += 2;
    } else {
        dim3 blk(32, 8);
        dim3 grd((g.ny + 31) / 32, (g.nx + 7) / 8);
        PC_CUDA_CHECK(cudaMemsetAsync(c->d_legacy_flags, 0, sizeof(uint32_t), s));
        legacy_flags2<T><<<grd, blk, 0, s>>>(a.Ein[0], a.Ein[1], a.Ein[2], g.nx, g.ny, g.pitch,
                                             c->d_legacy_flags);
        legacy_h2<T><<<grd, blk, 0, s>>>(a, c->d_legacy_flags);
        legacy_e2<T><<<grd, blk, 0, s>>>(a);
        c->launches += 3;
    }
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

int launch_legacy_step(pc_ctx* c, cudaStream_t s) {
    return c->g.precision == 8 ? legacy_step_t<double>(c, s) : legacy_step_t<float>(c, s);
}

template <typename T>
static int sources_t(pc_ctx* c, int row, cudaStream_t s) {
    const int ns = (int)c->sources.size();
    T* F[6];
    for (int q = 0; q < 6; ++q) F[q] = static_cast<T*>(c->F[c->cur][q]);
    for (int base = 0; base < ns; base += 32) {
        SrcLaunch L{};
        L.nsrc = ns - base < 32 ? ns - base : 32;
        int maxn = 1;
        for (int q = 0; q < L.nsrc; ++q) {
            const SourceDesc& d = c->sources[base + q];
            L.comp[q] = d.comp;
            L.n[q] = d.n;
            L.off[q] = d.d_off;
            L.w[q] = d.d_w;
            if (d.n > maxn) maxn = d.n;
        }
        dim3 grd((maxn + 255) / 256 < 64 ? (maxn + 255) / 256 : 64, L.nsrc);
        add_sources<T><<<grd, 256, 0, s>>>(L, F[0], F[1], F[2], F[3], F[4], F[5], c->d_amps,
                                           ns, row * ns + base);
        ++c->launches;
    }
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

int launch_sources(pc_ctx* c, int row, cudaStream_t s) {
    if (c->sources.empty()) return PC_OK;
    return c->g.precision == 8 ? sources_t<double>(c, row, s) : sources_t<float>(c, row, s);
}

}  // namespace pc
