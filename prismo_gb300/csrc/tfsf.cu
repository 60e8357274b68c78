// Plane-wave injection on a z = const plane fed by a 1D auxiliary grid (total-
// field / scattered-field).  The reference's TFSFSource (sources/tfsf.py:258-411)
// adds the incident field on one entry plane; this is the consistent form: the
// incident E and H come from a 1D Yee line with the same dz and dt, so for normal
// incidence the incident wave matches the 3D grid's own numerical dispersion.
//
// Per step (n -> n+1), with e1/h1 the auxiliary line and m0 its sample index:
//   after the H pass:  H_pol[k_H] += s_H Db e1[m0] / dz ;  h1 -= Db (e1[m] - e1[m-1]) / dz
//   after the E pass:  E_pol[k0]  += Cb   h1[m0] / dz ;  e1 -= Cb1 (h1[m+1] - h1[m]) / dz ;
//                      e1[0] = a(t_{n+1})
// k_H = k0 (+z) or k0+1 (-z); s_H = +1 for (x-pol, +z) and (y-pol, -z), else -1.
#include "pc_internal.cuh"

namespace pc {
namespace {

template <typename T>
__global__ void tfsf_h(T* H, const T* db_arr, T db_s, int nx, int ny, int pitch, int kH, int hcomp, T sgn,
                       const T* e1, int m0, T inv_dz, T* h1, int M) {
    // plane correction: one thread per (i, j)
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const T inc = e1[m0];  // incident E at time n (read before any e1 update)
    if (tid < nx * ny) {
        const int i = tid / ny, j = tid % ny;
        bool upd;
        if (hcomp == 4)  // Hy: updated for 1 <= i <= nx-2, j <= ny-2
            upd = i >= 1 && i <= nx - 2 && j <= ny - 2;
        else  // Hx: updated for i <= nx-2, 1 <= j <= ny-2
            upd = i <= nx - 2 && j >= 1 && j <= ny - 2;
        if (upd) {
            const int64_t o = ((int64_t)i * ny + j) * pitch + kH;
            const T db = db_arr ? db_arr[o] : db_s;
            H[o] += sgn * db * inc * inv_dz;
        }
    }
    // auxiliary line, H half step (reads e1, writes h1)
    for (int m = tid; m < M; m += gridDim.x * blockDim.x)
        if (m >= 1 && m <= M - 2) h1[m] -= db_s * (e1[m] - e1[m - 1]) * inv_dz;
}

template <typename T>
__global__ void tfsf_e(T* E, const T* cb, int nx, int ny, int pitch, int k0, int ecomp, const T* h1, int m0,
                       T inv_dz, T* e1, int M, T cb1, T amp) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const T inc = h1[m0];  // incident H at n+1/2
    if (tid < nx * ny) {
        const int i = tid / ny, j = tid % ny;
        const bool valid = ecomp == 0 ? (j <= ny - 2) : (i <= nx - 2);
        if (valid) {
            const int64_t o = ((int64_t)i * ny + j) * pitch + k0;
            E[o] += cb[o] * inc * inv_dz;
        }
    }
    for (int m = tid; m < M; m += gridDim.x * blockDim.x) {
        if (m == 0)
            e1[0] = amp;  // hard source at the head of the line
        else if (m <= M - 2)
            e1[m] -= cb1 * (h1[m + 1] - h1[m]) * inv_dz;
    }
}

template <typename T>
int tfsf_h_t(pc_ctx* c, cudaStream_t s) {
    const pc_grid_desc& g = c->g;
    const TfsfState& t = c->tfsf;
    const int hq = t.pol == 0 ? 4 : 3;  // Hy for x polarisation, Hx for y
    const int kH = t.dir > 0 ? t.k0 : t.k0 + 1;
    const T sgn = T(((t.pol == 0) == (t.dir > 0)) ? 1 : -1);
    const int n = g.nx * g.ny > t.M ? g.nx * g.ny : t.M;
    tfsf_h<T><<<(n + 255) / 256, 256, 0, s>>>(static_cast<T*>(c->F[c->cur][hq]),
                                              static_cast<const T*>(c->db[hq - 3]), T(c->db_s), g.nx, g.ny,
                                              g.pitch, kH, hq, sgn, static_cast<const T*>(t.d_e1), t.m0,
                                              T(1.0 / g.dz), static_cast<T*>(t.d_h1), t.M);
    ++c->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

template <typename T>
int tfsf_e_t(pc_ctx* c, double amp, cudaStream_t s) {
    const pc_grid_desc& g = c->g;
    const TfsfState& t = c->tfsf;
    const int eq = t.pol == 0 ? 0 : 1;
    const int n = g.nx * g.ny > t.M ? g.nx * g.ny : t.M;
    tfsf_e<T><<<(n + 255) / 256, 256, 0, s>>>(static_cast<T*>(c->F[c->cur][eq]), static_cast<const T*>(c->cb[eq]),
                                              g.nx, g.ny, g.pitch, t.k0, eq, static_cast<const T*>(t.d_h1), t.m0,
                                              T(1.0 / g.dz), static_cast<T*>(t.d_e1), t.M, T(t.cb1), T(amp));
    ++c->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

// The auxiliary line alone, one step, for the fused schedule (which applies the
// plane corrections inside its H + E kernel): inc[0] = e1[m0] at step n (the H
// correction), then the H half step, inc[1] = h1[m0] at n+1/2 (the E
// correction), then the E half step with the hard source.  The same arithmetic
// as tfsf_h / tfsf_e; one CTA, the two half steps separated by a barrier.
template <typename T>
__global__ void __launch_bounds__(1024) tfsf_line(T* e1, T* h1, int M, int m0, T db_s, T cb1, T inv_dz, T amp,
                                                  T* inc) {
    const int t = threadIdx.x;
    if (t == 0) inc[0] = e1[m0];
    for (int m = t; m < M; m += blockDim.x)
        if (m >= 1 && m <= M - 2) h1[m] -= db_s * (e1[m] - e1[m - 1]) * inv_dz;
    __syncthreads();
    if (t == 0) inc[1] = h1[m0];
    for (int m = t; m < M; m += blockDim.x) {
        if (m == 0)
            e1[0] = amp;
        else if (m <= M - 2)
            e1[m] -= cb1 * (h1[m + 1] - h1[m]) * inv_dz;
    }
}

template <typename T>
int tfsf_line_t(pc_ctx* c, double amp, cudaStream_t s) {
    const TfsfState& t = c->tfsf;
    tfsf_line<T><<<1, 1024, 0, s>>>(static_cast<T*>(t.d_e1), static_cast<T*>(t.d_h1), t.M, t.m0, T(c->db_s),
                                    T(t.cb1), T(1.0 / c->g.dz), T(amp), static_cast<T*>(t.d_inc));
    ++c->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

}  // namespace

int launch_tfsf_line(pc_ctx* c, double amp, cudaStream_t s) {
    if (!c->tfsf.on || !c->tfsf.d_inc) return PC_ERR_STATE;
    return c->g.precision == 8 ? tfsf_line_t<double>(c, amp, s) : tfsf_line_t<float>(c, amp, s);
}

int launch_tfsf_h(pc_ctx* c, cudaStream_t s) {
    return c->g.precision == 8 ? tfsf_h_t<double>(c, s) : tfsf_h_t<float>(c, s);
}

int launch_tfsf_e(pc_ctx* c, double amp, cudaStream_t s) {
    return c->g.precision == 8 ? tfsf_e_t<double>(c, amp, s) : tfsf_e_t<float>(c, amp, s);
}

}  // namespace pc
