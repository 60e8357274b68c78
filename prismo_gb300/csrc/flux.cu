// Plane monitors: power through a plane (flux) and mode-expansion coefficients,
// in time and in frequency.
//
// monitors/flux.py:126-173 sums S_n = (E x H)_n over the monitor surface times the
// cell area every step, and :219-285 forms P(w) = 1/2 Re sum (E x H*)_n dA from
// the DFTs of the fields; both take the field values at the same index for every
// component.  The reference's region is a fixed [:10, :10] placeholder
// (flux.py:104-106, 187-191); here the plane is the monitor's real region, the
// components' common index range.
//
// Time domain: one CTA per plane after every step gathers the four tangential
// components, reduces in float64 and appends to the history at a device counter
// (so a replayed graph of steps appends in order).  Frequency domain: the four
// components' DFT monitors (dft.cu) are flushed and one CTA per frequency reduces
// their accumulators.
//
// Mode expansion (monitors/mode_monitor.py:137-199 with
// utils/mode_matching.py:41-131): a_m(t) = 1/2 sum (E x H_m* + E_m* x H)_n / P_m is a
// linear function of the four tangential fields on the plane with complex weights
// from the mode profile, which the host builds; one CTA per plane reduces every
// mode after every step into a complex history at a device counter, and the
// spectrum sum_n a_m(t_n) exp(-i w t_n) dt (mode_monitor.py:171-175) is formed
// from that history when it is read.
#include "pc_internal.cuh"

namespace pc {
namespace {

constexpr int FLUX_THREADS = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    v = threadIdx.x < FLUX_THREADS / 32 ? sh[threadIdx.x] : 0.0;
    if (warp == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__global__ void __launch_bounds__(FLUX_THREADS) flux_sample(const T* f0, const T* f1, const T* f2, const T* f3,
                                                           const int64_t* __restrict__ off, int npts, double scale,
                                                           double* hist, int64_t* count, int64_t capacity) {
    __shared__ double sh[FLUX_THREADS / 32];
    double acc = 0.0;
    for (int p = threadIdx.x; p < npts; p += FLUX_THREADS) {
        const double a = (double)f0[off[p]] * (double)f1[off[npts + p]];
        const double b = (double)f2[off[2 * npts + p]] * (double)f3[off[3 * npts + p]];
        acc += a - b;
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) {
        const int64_t n = *count;
        if (n < capacity) hist[n] = acc * scale;
        *count = n + 1;
    }
}

// P(f) = 1/2 Re sum_p (A B* - C D*) * scale from four DFT accumulators
// (float4: running sum re, im and their Kahan compensations).
__global__ void __launch_bounds__(FLUX_THREADS) flux_spectrum(const float4* a, const float4* b, const float4* c,
                                                             const float4* d, int npts, double scale, double* out) {
    __shared__ double sh[FLUX_THREADS / 32];
    const int f = blockIdx.x;
    auto val = [&](const float4* x, int p, double& re, double& im) {
        const float4 v = x[(int64_t)f * npts + p];
        re = (double)v.x - (double)v.z;
        im = (double)v.y - (double)v.w;
    };
    double acc = 0.0;
    for (int p = threadIdx.x; p < npts; p += FLUX_THREADS) {
        double ar, ai, br, bi, cr, ci, dr, di;
        val(a, p, ar, ai);
        val(b, p, br, bi);
        val(c, p, cr, ci);
        val(d, p, dr, di);
        acc += (ar * br + ai * bi) - (cr * dr + ci * di);  // Re(A B*) - Re(C D*)
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) out[f] = 0.5 * acc * scale;
}

template <typename T>
__global__ void __launch_bounds__(FLUX_THREADS) mode_sample(const T* f0, const T* f1, const T* f2, const T* f3,
                                                           const int64_t* __restrict__ off,
                                                           const double2* __restrict__ w, int npts, int nmodes,
                                                           double2* hist, int64_t* count, int64_t capacity) {
    __shared__ double sh[FLUX_THREADS / 32];
    const int64_t n = *count;
    for (int m = 0; m < nmodes; ++m) {
        const double2* wm = w + (int64_t)m * 4 * npts;
        double re = 0.0, im = 0.0;
        for (int p = threadIdx.x; p < npts; p += FLUX_THREADS) {
            const double v0 = (double)f0[off[p]], v1 = (double)f1[off[npts + p]];
            const double v2 = (double)f2[off[2 * npts + p]], v3 = (double)f3[off[3 * npts + p]];
            const double2 a = wm[p], b = wm[npts + p], c = wm[2 * npts + p], d = wm[3 * npts + p];
            re += a.x * v0 + b.x * v1 + c.x * v2 + d.x * v3;
            im += a.y * v0 + b.y * v1 + c.y * v2 + d.y * v3;
        }
        re = block_sum(re, sh);
        __syncthreads();  // sh is reused
        im = block_sum(im, sh);
        __syncthreads();
        if (threadIdx.x == 0 && n < capacity) hist[n * nmodes + m] = make_double2(re, im);
    }
    if (threadIdx.x == 0) *count = n + 1;
}

// Mode ports (boundaries/mode_port.py:261-429): F[off[p]] += amp w[p] in float64,
// rounded once to the field type (NumPy's in-place add of a float64 product), and
// a one-shot complex weighted sum over the port plane for the extraction.
template <typename T>
__global__ void scatter_add(T* f, const int64_t* __restrict__ off, const double* __restrict__ w, int64_t n,
                            double amp) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        f[off[i]] = (T)__dadd_rn((double)f[off[i]], __dmul_rn(amp, w[i]));  // no contraction into an FMA
}

template <typename T>
__global__ void __launch_bounds__(FLUX_THREADS) plane_overlap(const T* f0, const T* f1, const T* f2, const T* f3,
                                                             const int64_t* __restrict__ off,
                                                             const double2* __restrict__ w, int npts, int nmodes,
                                                             double2* out) {
    __shared__ double sh[FLUX_THREADS / 32];
    const int m = blockIdx.x;
    const double2* wm = w + (int64_t)m * 4 * npts;
    double re = 0.0, im = 0.0;
    for (int p = threadIdx.x; p < npts; p += FLUX_THREADS) {
        const double v[4] = {(double)f0[off[p]], (double)f1[off[npts + p]], (double)f2[off[2 * npts + p]],
                             (double)f3[off[3 * npts + p]]};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double2 a = wm[(int64_t)q * npts + p];
            re += a.x * v[q];
            im += a.y * v[q];
        }
    }
    re = block_sum(re, sh);
    __syncthreads();
    im = block_sum(im, sh);
    if (threadIdx.x == 0 && m < nmodes) out[m] = make_double2(re, im);
}

// out[m][f] = sum_{n < nsteps} hist[n][m] exp(-i w_f (t0 + n dt)) dt
__global__ void __launch_bounds__(FLUX_THREADS) mode_spectrum(const double2* __restrict__ hist, int64_t nsteps,
                                                             int nmodes, const double* __restrict__ omega, int nf,
                                                             double t0, double dt, double2* out) {
    __shared__ double sh[FLUX_THREADS / 32];
    const int f = blockIdx.x, m = blockIdx.y;
    double re = 0.0, im = 0.0;
    for (int64_t n = threadIdx.x; n < nsteps; n += FLUX_THREADS) {
        double s, c;
        sincos(-omega[f] * (t0 + (double)n * dt), &s, &c);
        const double2 a = hist[n * nmodes + m];
        re += a.x * c - a.y * s;
        im += a.x * s + a.y * c;
    }
    re = block_sum(re, sh);
    __syncthreads();
    im = block_sum(im, sh);
    if (threadIdx.x == 0) out[(int64_t)m * nf + f] = make_double2(re * dt, im * dt);
}

}  // namespace

int mode_after_step(pc_ctx* c, cudaStream_t s) {
    for (auto& m : c->modes) {
        if (c->g.precision == 8) {
            auto F = [&](int q) { return static_cast<const double*>(c->F[c->cur][m.comp[q]]); };
            mode_sample<double><<<1, FLUX_THREADS, 0, s>>>(F(0), F(1), F(2), F(3), m.d_off, m.d_w, m.npts, m.nmodes,
                                                           m.d_hist, m.d_count, m.capacity);
        } else {
            auto F = [&](int q) { return static_cast<const float*>(c->F[c->cur][m.comp[q]]); };
            mode_sample<float><<<1, FLUX_THREADS, 0, s>>>(F(0), F(1), F(2), F(3), m.d_off, m.d_w, m.npts, m.nmodes,
                                                          m.d_hist, m.d_count, m.capacity);
        }
        ++c->launches;
    }
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

void mode_monitor_free(ModeMonitor& m) {
    cudaFree(m.d_off);
    cudaFree(m.d_w);
    cudaFree(m.d_count);
    cudaFree(m.d_omega);
    m.d_off = nullptr;
    m.d_w = nullptr;
    m.d_count = nullptr;
    m.d_omega = nullptr;
}

int flux_after_step(pc_ctx* c, cudaStream_t s) {
    for (auto& m : c->fluxes) {
        const int64_t n = m.npts;
        if (c->g.precision == 8) {
            auto F = [&](int q) { return static_cast<const double*>(c->F[c->cur][m.comp[q]]); };
            flux_sample<double><<<1, FLUX_THREADS, 0, s>>>(F(0), F(1), F(2), F(3), m.d_off, (int)n, m.scale,
                                                           m.d_hist, m.d_count, m.capacity);
        } else {
            auto F = [&](int q) { return static_cast<const float*>(c->F[c->cur][m.comp[q]]); };
            flux_sample<float><<<1, FLUX_THREADS, 0, s>>>(F(0), F(1), F(2), F(3), m.d_off, (int)n, m.scale,
                                                          m.d_hist, m.d_count, m.capacity);
        }
        ++c->launches;
    }
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

void flux_monitor_free(FluxMonitor& m) {
    cudaFree(m.d_off);
    cudaFree(m.d_count);
    m.d_off = nullptr;
    m.d_count = nullptr;
}

}  // namespace pc

using namespace pc;

int pc_add_flux(pc_ctx* c, const int32_t comps[4], const int64_t* offsets, int32_t npts, double scale, double* d_hist,
                int64_t capacity) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c || !comps || !offsets || npts <= 0 || !d_hist || capacity <= 0) return PC_ERR_INVALID;
    for (int q = 0; q < 4; ++q)
        if (comps[q] < 0 || comps[q] > 5) return PC_ERR_INVALID;
    const int64_t limit = (int64_t)c->g.nx * c->g.ny * c->g.pitch;
    for (int64_t i = 0; i < 4 * (int64_t)npts; ++i)
        if (offsets[i] < 0 || offsets[i] >= limit) return PC_ERR_INVALID;
    FluxMonitor m{};
    for (int q = 0; q < 4; ++q) m.comp[q] = comps[q];
    m.npts = npts;
    m.scale = scale;
    m.d_hist = d_hist;
    m.capacity = capacity;
    bool ok = cudaMalloc(&m.d_off, 4 * (size_t)npts * sizeof(int64_t)) == cudaSuccess &&
              cudaMalloc(&m.d_count, sizeof(int64_t)) == cudaSuccess;
    ok = ok && cudaMemcpy(m.d_off, offsets, 4 * (size_t)npts * sizeof(int64_t), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(m.d_count, 0, sizeof(int64_t)) == cudaSuccess;
    if (!ok) {
        flux_monitor_free(m);
        return PC_ERR_CUDA;
    }
    c->fluxes.push_back(m);
    return (int)c->fluxes.size() - 1;
}

int pc_flux_count(pc_ctx* c, int32_t id, int64_t* count, void* stream) {
    if (!c || !count || id < 0 || id >= (int)c->fluxes.size()) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    PC_CUDA_CHECK(cudaMemcpyAsync(count, c->fluxes[id].d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    PC_CUDA_CHECK(cudaStreamSynchronize(s));
    return PC_OK;
}

int pc_flux_spectrum(pc_ctx* c, const int32_t dft_ids[4], double scale, double* d_out, void* stream) {
    if (!c || !dft_ids || !d_out) return PC_ERR_INVALID;
    const int nd = (int)c->dfts.size();
    for (int q = 0; q < 4; ++q)
        if (dft_ids[q] < 0 || dft_ids[q] >= nd) return PC_ERR_INVALID;
    const DftMonitor& m0 = c->dfts[dft_ids[0]];
    for (int q = 1; q < 4; ++q)
        if (c->dfts[dft_ids[q]].npts != m0.npts || c->dfts[dft_ids[q]].nf != m0.nf) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    for (int q = 0; q < 4; ++q) {
        const int rc = dft_flush_monitor(c, c->dfts[dft_ids[q]], s);
        if (rc) return rc;
    }
    flux_spectrum<<<m0.nf, FLUX_THREADS, 0, s>>>(c->dfts[dft_ids[0]].d_acc, c->dfts[dft_ids[1]].d_acc,
                                                 c->dfts[dft_ids[2]].d_acc, c->dfts[dft_ids[3]].d_acc, m0.npts, scale,
                                                 d_out);
    ++c->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

int pc_add_mode_monitor(pc_ctx* c, const int32_t comps[4], const int64_t* offsets, int32_t npts, int32_t nmodes,
                        const double* weights, void* d_hist, int64_t capacity) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c || !comps || !offsets || npts <= 0 || nmodes <= 0 || nmodes > 64 || !weights || !d_hist || capacity <= 0)
        return PC_ERR_INVALID;
    for (int q = 0; q < 4; ++q)
        if (comps[q] < 0 || comps[q] > 5) return PC_ERR_INVALID;
    const int64_t limit = (int64_t)c->g.nx * c->g.ny * c->g.pitch;
    for (int64_t i = 0; i < 4 * (int64_t)npts; ++i)
        if (offsets[i] < 0 || offsets[i] >= limit) return PC_ERR_INVALID;
    ModeMonitor m{};
    for (int q = 0; q < 4; ++q) m.comp[q] = comps[q];
    m.npts = npts;
    m.nmodes = nmodes;
    m.d_hist = static_cast<double2*>(d_hist);
    m.capacity = capacity;
    const size_t nw = (size_t)nmodes * 4 * npts;
    bool ok = cudaMalloc(&m.d_off, 4 * (size_t)npts * sizeof(int64_t)) == cudaSuccess &&
              cudaMalloc(&m.d_w, nw * sizeof(double2)) == cudaSuccess &&
              cudaMalloc(&m.d_count, sizeof(int64_t)) == cudaSuccess;
    ok = ok && cudaMemcpy(m.d_off, offsets, 4 * (size_t)npts * sizeof(int64_t), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(m.d_w, weights, nw * sizeof(double2), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(m.d_count, 0, sizeof(int64_t)) == cudaSuccess;
    if (!ok) {
        mode_monitor_free(m);
        return PC_ERR_CUDA;
    }
    c->modes.push_back(m);
    return (int)c->modes.size() - 1;
}

int pc_mode_count(pc_ctx* c, int32_t id, int64_t* count, void* stream) {
    if (!c || !count || id < 0 || id >= (int)c->modes.size()) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    PC_CUDA_CHECK(cudaMemcpyAsync(count, c->modes[id].d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    PC_CUDA_CHECK(cudaStreamSynchronize(s));
    return PC_OK;
}

int pc_mode_spectrum(pc_ctx* c, int32_t id, const double* omega, int32_t nf, double t0, double dt, void* d_out,
                     void* stream) {
    if (!c || id < 0 || id >= (int)c->modes.size() || !omega || nf <= 0 || !d_out) return PC_ERR_INVALID;
    ModeMonitor& m = c->modes[id];
    int64_t n = 0;
    const int rc = pc_mode_count(c, id, &n, stream);
    if (rc) return rc;
    if (n > m.capacity) return PC_ERR_STATE;  // the history lost steps
    cudaStream_t s = (cudaStream_t)stream;
    if (nf > m.omega_cap) {
        cudaFree(m.d_omega);
        m.d_omega = nullptr;
        m.omega_cap = 0;
        PC_CUDA_CHECK(cudaMalloc(&m.d_omega, nf * sizeof(double)));
        m.omega_cap = nf;
    }
    PC_CUDA_CHECK(cudaMemcpyAsync(m.d_omega, omega, nf * sizeof(double), cudaMemcpyHostToDevice, s));
    mode_spectrum<<<dim3(nf, m.nmodes), FLUX_THREADS, 0, s>>>(m.d_hist, n, m.nmodes, m.d_omega, nf, t0, dt,
                                                             static_cast<double2*>(d_out));
    ++c->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    PC_CUDA_CHECK(cudaStreamSynchronize(s));  // the omega copy's host buffer is the caller's
    return PC_OK;
}

int pc_scatter_add(int32_t precision, void* field, const int64_t* d_off, const double* d_w, int64_t n, double amp,
                   void* stream) {
    if ((precision != 4 && precision != 8) || !field || !d_off || !d_w || n < 0) return PC_ERR_INVALID;
    if (n == 0) return PC_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    if (precision == 8)
        scatter_add<double><<<blocks, 256, 0, s>>>(static_cast<double*>(field), d_off, d_w, n, amp);
    else
        scatter_add<float><<<blocks, 256, 0, s>>>(static_cast<float*>(field), d_off, d_w, n, amp);
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

int pc_plane_overlap(int32_t precision, const void* const fields[4], const int64_t* d_off, int32_t npts,
                     int32_t nmodes, const void* d_w, void* d_out, void* stream) {
    if ((precision != 4 && precision != 8) || !fields || !d_off || !d_w || !d_out || npts <= 0 || nmodes <= 0)
        return PC_ERR_INVALID;
    for (int q = 0; q < 4; ++q)
        if (!fields[q]) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const double2* w = static_cast<const double2*>(d_w);
    double2* out = static_cast<double2*>(d_out);
    if (precision == 8)
        plane_overlap<double><<<nmodes, FLUX_THREADS, 0, s>>>(
            static_cast<const double*>(fields[0]), static_cast<const double*>(fields[1]),
            static_cast<const double*>(fields[2]), static_cast<const double*>(fields[3]), d_off, w, npts, nmodes, out);
    else
        plane_overlap<float><<<nmodes, FLUX_THREADS, 0, s>>>(
            static_cast<const float*>(fields[0]), static_cast<const float*>(fields[1]),
            static_cast<const float*>(fields[2]), static_cast<const float*>(fields[3]), d_off, w, npts, nmodes, out);
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}
