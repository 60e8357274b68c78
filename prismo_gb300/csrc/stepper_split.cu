// Corrected Yee stepper, split schedule: one H pass and one E pass per step,
// in place, with the CPML psi recursions fused into the curl terms.
//
// Update rules (3D; 2D in the *_2 kernels):
//   Hx[:, 1:-1, 1:-1] = Da Hx - Db ((kinv_y dEz/dy + psi_Hxy) - (kinv_z dEy/dz + psi_Hxz))
//   Hy[1:-1, :, 1:-1] = Da Hy - Db ((kinv_z dEx/dz + psi_Hyz) - (kinv_x dEz/dx + psi_Hyx))
//   Hz[1:-1, 1:-1, :] = Da Hz - Db ((kinv_x dEy/dx + psi_Hzx) - (kinv_y dEx/dy + psi_Hzy))
//   Ex = Ca Ex + Cb ((kinv_y dHz/dy + psi_Exy) - (kinv_z dHy/dz + psi_Exz))   (etc.)
// with backward differences of E and forward differences of H.  These are the
// reference curls (core/solver.py:167-309) with H written one index later, which
// makes the discrete curl pair adjoint; psi <- b psi + a d is the Roden-Gedney
// recursion with the boundaries/pml.py:117-257 profiles.  The E passes set
// PC_STATUS_NONFINITE in the status word when a value they write is NaN or Inf.
#include <algorithm>

#include "pc_internal.cuh"
#include "stencil_common.cuh"

namespace pc {
namespace {

template <typename T, bool CPML>
__global__ void __launch_bounds__(256) split_h3(FieldArgs<T> a, CpmlArgs<T> p) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (k >= nz || j >= ny) return;
    const int64_t P = a.pitch, R = (int64_t)ny * P;
    const int64_t o = ((int64_t)i * ny + j) * P + k;
    const T *Ex = a.Ein[0], *Ey = a.Ein[1], *Ez = a.Ein[2];
    T *Hx = a.Hout[0], *Hy = a.Hout[1], *Hz = a.Hout[2];
    const Idx3 q{i, j, k, nx, ny, nz, a.pitch};
    if (i < nx - 1 && j >= 1 && j <= ny - 2 && k >= 1 && k <= nz - 2) {
        T cy = (Ez[o] - Ez[o - P]) * a.inv_dy;
        T cz = (Ey[o] - Ey[o - 1]) * a.inv_dz;
        if (CPML) {
            cy = cpml3<T, 1>(p, SY_HX, q, cy);
            cz = cpml3<T, 2>(p, SZ_HX, q, cz);
        }
        Hx[o] = hcoef(a.da[0], o, a.da_s) * Hx[o] - hcoef(a.db[0], o, a.db_s) * (cy - cz);
    }
    if (i >= 1 && i <= nx - 2 && j < ny - 1 && k >= 1 && k <= nz - 2) {
        T cz = (Ex[o] - Ex[o - 1]) * a.inv_dz;
        T cx = (Ez[o] - Ez[o - R]) * a.inv_dx;
        if (CPML) {
            cz = cpml3<T, 2>(p, SZ_HY, q, cz);
            cx = cpml3<T, 0>(p, SX_HY, q, cx);
        }
        Hy[o] = hcoef(a.da[1], o, a.da_s) * Hy[o] - hcoef(a.db[1], o, a.db_s) * (cz - cx);
    }
    if (i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2 && k < nz - 1) {
        T cx = (Ey[o] - Ey[o - R]) * a.inv_dx;
        T cy = (Ex[o] - Ex[o - P]) * a.inv_dy;
        if (CPML) {
            cx = cpml3<T, 0>(p, SX_HZ, q, cx);
            cy = cpml3<T, 1>(p, SY_HZ, q, cy);
        }
        Hz[o] = hcoef(a.da[2], o, a.da_s) * Hz[o] - hcoef(a.db[2], o, a.db_s) * (cx - cy);
    }
}

template <typename T, bool CPML, bool ADE>
__global__ void __launch_bounds__(256) split_e3(FieldArgs<T> a, CpmlArgs<T> p, AdeArgs<T> ade) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (k >= nz || j >= ny) return;
    const int64_t P = a.pitch, R = (int64_t)ny * P;
    const int64_t o = ((int64_t)i * ny + j) * P + k;
    const T *Hx = a.Hin[0], *Hy = a.Hin[1], *Hz = a.Hin[2];
    T *Ex = a.Eout[0], *Ey = a.Eout[1], *Ez = a.Eout[2];
    const Idx3 q{i, j, k, nx, ny, nz, a.pitch};
    T chk = T(0);  // non-finite sentinel: the sum of the values this thread wrote
    if (j < ny - 1 && k < nz - 1) {
        T c1 = (Hz[o + P] - Hz[o]) * a.inv_dy;
        T c2 = (Hy[o + 1] - Hy[o]) * a.inv_dz;
        if (CPML) {
            c1 = cpml3<T, 1>(p, SY_EX, q, c1);
            c2 = cpml3<T, 2>(p, SZ_EX, q, c2);
        }
        T e = Ex[o];
        if (!(ADE && ade_update(ade, 0, i, j, k, c1 - c2, e))) e = ecoef(a.ca[0], o) * e + a.cb[0][o] * (c1 - c2);
        Ex[o] = e;
        chk += e;
    }
    if (i < nx - 1 && k < nz - 1) {
        T c1 = (Hx[o + 1] - Hx[o]) * a.inv_dz;
        T c2 = (Hz[o + R] - Hz[o]) * a.inv_dx;
        if (CPML) {
            c1 = cpml3<T, 2>(p, SZ_EY, q, c1);
            c2 = cpml3<T, 0>(p, SX_EY, q, c2);
        }
        T e = Ey[o];
        if (!(ADE && ade_update(ade, 1, i, j, k, c1 - c2, e))) e = ecoef(a.ca[1], o) * e + a.cb[1][o] * (c1 - c2);
        Ey[o] = e;
        chk += e;
    }
    if (i < nx - 1 && j < ny - 1) {
        T c1 = (Hy[o + R] - Hy[o]) * a.inv_dx;
        T c2 = (Hx[o + P] - Hx[o]) * a.inv_dy;
        if (CPML) {
            c1 = cpml3<T, 0>(p, SX_EZ, q, c1);
            c2 = cpml3<T, 1>(p, SY_EZ, q, c2);
        }
        T e = Ez[o];
        if (!(ADE && ade_update(ade, 2, i, j, k, c1 - c2, e))) e = ecoef(a.ca[2], o) * e + a.cb[2][o] * (c1 - c2);
        Ez[o] = e;
        chk += e;
    }
    if (!isfinite(chk)) atomicOr(a.status, PC_STATUS_NONFINITE);
}

// 2D: both families (Ez, Hx, Hy) and (Hz, Ex, Ey); layout i * pitch + j.
template <typename T, bool CPML>
__global__ void __launch_bounds__(256) split_h2(FieldArgs<T> a, CpmlArgs<T> p) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int nx = a.nx, ny = a.ny;
    if (i >= nx || j >= ny) return;
    const int64_t P = a.pitch;
    const int64_t o = (int64_t)i * P + j;
    const T *Ex = a.Ein[0], *Ey = a.Ein[1], *Ez = a.Ein[2];
    T *Hx = a.Hout[0], *Hy = a.Hout[1], *Hz = a.Hout[2];
    const Idx2 q{i, j, nx, ny, a.pitch};
    if (i < nx - 1 && j >= 1 && j <= ny - 2) {
        T cy = (Ez[o] - Ez[o - 1]) * a.inv_dy;
        if (CPML) cy = cpml2<T, 1>(p, SY_HX, q, cy);
        Hx[o] = hcoef(a.da[0], o, a.da_s) * Hx[o] - hcoef(a.db[0], o, a.db_s) * cy;
    }
    if (i >= 1 && i <= nx - 2 && j < ny - 1) {
        T cx = (Ez[o] - Ez[o - P]) * a.inv_dx;
        if (CPML) cx = cpml2<T, 0>(p, SX_HY, q, cx);
        Hy[o] = hcoef(a.da[1], o, a.da_s) * Hy[o] + hcoef(a.db[1], o, a.db_s) * cx;
    }
    if (i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2) {
        T cx = (Ey[o] - Ey[o - P]) * a.inv_dx;
        T cy = (Ex[o] - Ex[o - 1]) * a.inv_dy;
        if (CPML) {
            cx = cpml2<T, 0>(p, SX_HZ, q, cx);
            cy = cpml2<T, 1>(p, SY_HZ, q, cy);
        }
        Hz[o] = hcoef(a.da[2], o, a.da_s) * Hz[o] - hcoef(a.db[2], o, a.db_s) * (cx - cy);
    }
}

template <typename T, bool CPML, bool ADE>
__global__ void __launch_bounds__(256) split_e2(FieldArgs<T> a, CpmlArgs<T> p, AdeArgs<T> ade) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int nx = a.nx, ny = a.ny;
    if (i >= nx || j >= ny) return;
    const int64_t P = a.pitch;
    const int64_t o = (int64_t)i * P + j;
    const T *Hx = a.Hin[0], *Hy = a.Hin[1], *Hz = a.Hin[2];
    T *Ex = a.Eout[0], *Ey = a.Eout[1], *Ez = a.Eout[2];
    const Idx2 q{i, j, nx, ny, a.pitch};
    T chk = T(0);  // non-finite sentinel: the sum of the values this thread wrote
    if (i < nx - 1 && j < ny - 1) {
        T c1 = (Hy[o + P] - Hy[o]) * a.inv_dx;
        T c2 = (Hx[o + 1] - Hx[o]) * a.inv_dy;
        if (CPML) {
            c1 = cpml2<T, 0>(p, SX_EZ, q, c1);
            c2 = cpml2<T, 1>(p, SY_EZ, q, c2);
        }
        T e = Ez[o];
        if (!(ADE && ade_update(ade, 2, i, j, 0, c1 - c2, e))) e = ecoef(a.ca[2], o) * e + a.cb[2][o] * (c1 - c2);
        Ez[o] = e;
        chk += e;
    }
    if (j < ny - 1) {
        T c = (Hz[o + 1] - Hz[o]) * a.inv_dy;
        if (CPML) c = cpml2<T, 1>(p, SY_EX, q, c);
        T e = Ex[o];
        if (!(ADE && ade_update(ade, 0, i, j, 0, c, e))) e = ecoef(a.ca[0], o) * e + a.cb[0][o] * c;
        Ex[o] = e;
        chk += e;
    }
    if (i < nx - 1) {
        T c = (Hz[o + P] - Hz[o]) * a.inv_dx;
        if (CPML) c = cpml2<T, 0>(p, SX_EY, q, c);
        T e = Ey[o];
        if (!(ADE && ade_update(ade, 1, i, j, 0, -c, e))) e = ecoef(a.ca[1], o) * e - a.cb[1][o] * c;
        Ey[o] = e;
        chk += e;
    }
    if (!isfinite(chk)) atomicOr(a.status, PC_STATUS_NONFINITE);
}

// The pole terms of the ADE E update on the fused schedule.  The fused H + E
// kernel stored the partial value ce E^n + inv (dt/eps0) curl (ade_partial) at
// every point of the dispersive regions in the output set; this pass subtracts
// the poles' terms, advances the auxiliaries and stores E^{n+1}, reading E^n from
// the input set.  Same update ranges per component as split_e3 and the same
// arithmetic as ade_poles; a point in several boxes belongs to the first
// (ade_region_of).  Every load of a point is issued before the first store, so a
// thread keeps up to 3 x (2 + 2 PC_MAX_ADE_POLES) loads in flight (the stores to
// the auxiliaries could alias later loads if they were interleaved).
template <typename T>
__global__ void __launch_bounds__(256) ade_pass3(FieldArgs<T> a, AdeArgs<T> A, int r, KernelDft<T> D) {
    const int* b = A.box[r];
    const int k = b[4] + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = b[2] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = b[0] + blockIdx.z;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (k >= b[5] || j >= b[3] || i >= b[1] || k >= nz || j >= ny || i >= nx) return;
    if (ade_region_of(A, i, j, k) != r) return;
    const int64_t o = ((int64_t)i * ny + j) * a.pitch + k;
    const int64_t ao = ade_offset(A, r, i, j, k);
    const bool upd[3] = {j < ny - 1 && k < nz - 1, i < nx - 1 && k < nz - 1, i < nx - 1 && j < ny - 1};
    const int np = A.npoles[r];
    T e0[3], acc[3], x0[3][PC_MAX_ADE_POLES], x1[3][PC_MAX_ADE_POLES];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        e0[c] = acc[c] = T(0);
#pragma unroll
        for (int p = 0; p < PC_MAX_ADE_POLES; ++p) x0[c][p] = x1[c][p] = T(0);
        if (!upd[c]) continue;
        e0[c] = a.Ein[c][o];
        acc[c] = a.Eout[c][o];
#pragma unroll
        for (int p = 0; p < PC_MAX_ADE_POLES; ++p) {
            if (p >= np) break;
            x0[c][p] = A.aux[r][c][p][0][ao];
            if (A.kind[r][p] == 0) x1[c][p] = A.aux[r][c][p][1][ao];
        }
    }
    const T inv = A.inv[r];
    T chk = T(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (!upd[c]) continue;
        T e = acc[c];
#pragma unroll
        for (int p = 0; p < PC_MAX_ADE_POLES; ++p) {
            if (p >= np) break;
            if (A.kind[r][p] == 0)
                e -= inv * (A.c2[r][p] * x0[c][p] - A.c3[r][p] * x1[c][p]);
            else if (A.kind[r][p] == 1)
                e -= inv * (T(0.5) * A.dt * (T(1) + A.c1[r][p]) * x0[c][p]);
            else
                e -= inv * ((A.c1[r][p] - T(1)) * x0[c][p]);
        }
#pragma unroll
        for (int p = 0; p < PC_MAX_ADE_POLES; ++p) {
            if (p >= np) break;
            if (A.kind[r][p] == 0) {
                const T dn = (A.c0[r][p] * e + A.c1[r][p] * e0[c]) + (A.c2[r][p] * x0[c][p] - A.c3[r][p] * x1[c][p]);
                A.aux[r][c][p][1][ao] = dn;
                A.aux[r][c][p][0][ao] = x0[c][p] + dn;
            } else {
                A.aux[r][c][p][0][ao] = A.c1[r][p] * x0[c][p] + A.c0[r][p] * (T(0.5) * (e + e0[c]));
            }
        }
        a.Eout[c][o] = e;
        chk += e;
#pragma unroll
        for (int m = 0; m < PC_MAX_FUSED_DFT; ++m)  // plane DFT samples of the final E
            if (m < D.n && D.comp[m] == c && k == D.k[m] && i < D.nx[m] && j < D.ny[m])
                D.row[m][(int64_t)i * D.ny[m] + j] = static_cast<float>(e);
    }
    if (!isfinite(chk)) atomicOr(a.status, PC_STATUS_NONFINITE);
}

// ade_pass3 with V consecutive k points per thread (float2 accesses for V = 2):
// for a single region whose k range starts and ends on multiples of V and ends
// before the last k (so every component's update range is uniform over the V
// points, and region ownership needs no per-point test).  Same arithmetic.
template <typename T, int V>
struct VecOf;
template <>
struct VecOf<float, 2> {
    using type = float2;
};

template <typename T, int V>
__global__ void __launch_bounds__(256) ade_pass3v(FieldArgs<T> a, AdeArgs<T> A, KernelDft<T> D) {
    using VT = typename VecOf<T, V>::type;
    const int* b = A.box[0];
    const int k = b[4] + (int)(blockIdx.x * blockDim.x + threadIdx.x) * V;
    const int j = b[2] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = b[0] + blockIdx.z;
    const int nx = a.nx, ny = a.ny;
    if (k >= b[5] || j >= b[3] || i >= b[1] || j >= ny || i >= nx) return;
    const int64_t o = ((int64_t)i * ny + j) * a.pitch + k;
    const int64_t ao = ade_offset(A, 0, i, j, k);
    const bool upd[3] = {j < ny - 1, i < nx - 1, i < nx - 1 && j < ny - 1};
    const int np = A.npoles[0];
    T e0[3][V], acc[3][V], x0[3][PC_MAX_ADE_POLES][V], x1[3][PC_MAX_ADE_POLES][V];
    auto ld = [&](const T* p, T* v) {
        const VT w = *reinterpret_cast<const VT*>(p);
        const T* q = reinterpret_cast<const T*>(&w);
#pragma unroll
        for (int l = 0; l < V; ++l) v[l] = q[l];
    };
    auto st = [&](T* p, const T* v) {
        VT w;
        T* q = reinterpret_cast<T*>(&w);
#pragma unroll
        for (int l = 0; l < V; ++l) q[l] = v[l];
        *reinterpret_cast<VT*>(p) = w;
    };
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (!upd[c]) continue;
        ld(a.Ein[c] + o, e0[c]);
        ld(a.Eout[c] + o, acc[c]);
#pragma unroll
        for (int p = 0; p < PC_MAX_ADE_POLES; ++p) {
            if (p >= np) break;
            ld(A.aux[0][c][p][0] + ao, x0[c][p]);
            if (A.kind[0][p] == 0) ld(A.aux[0][c][p][1] + ao, x1[c][p]);
        }
    }
    const T inv = A.inv[0];
    T chk = T(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (!upd[c]) continue;
        T e[V];
#pragma unroll
        for (int l = 0; l < V; ++l) {
            T v = acc[c][l];
#pragma unroll
            for (int p = 0; p < PC_MAX_ADE_POLES; ++p) {
                if (p >= np) break;
                if (A.kind[0][p] == 0)
                    v -= inv * (A.c2[0][p] * x0[c][p][l] - A.c3[0][p] * x1[c][p][l]);
                else if (A.kind[0][p] == 1)
                    v -= inv * (T(0.5) * A.dt * (T(1) + A.c1[0][p]) * x0[c][p][l]);
                else
                    v -= inv * ((A.c1[0][p] - T(1)) * x0[c][p][l]);
            }
            e[l] = v;
            chk += v;
        }
#pragma unroll
        for (int p = 0; p < PC_MAX_ADE_POLES; ++p) {
            if (p >= np) break;
            T n0[V], n1[V];
#pragma unroll
            for (int l = 0; l < V; ++l) {
                if (A.kind[0][p] == 0) {
                    n1[l] = (A.c0[0][p] * e[l] + A.c1[0][p] * e0[c][l]) +
                            (A.c2[0][p] * x0[c][p][l] - A.c3[0][p] * x1[c][p][l]);
                    n0[l] = x0[c][p][l] + n1[l];
                } else {
                    n0[l] = A.c1[0][p] * x0[c][p][l] + A.c0[0][p] * (T(0.5) * (e[l] + e0[c][l]));
                }
            }
            if (A.kind[0][p] == 0) st(A.aux[0][c][p][1] + ao, n1);
            st(A.aux[0][c][p][0] + ao, n0);
        }
        st(a.Eout[c] + o, e);
#pragma unroll
        for (int m = 0; m < PC_MAX_FUSED_DFT; ++m)  // plane DFT samples of the final E
            if (m < D.n && D.comp[m] == c && i < D.nx[m] && j < D.ny[m]) {
#pragma unroll
                for (int l = 0; l < V; ++l)
                    if (k + l == D.k[m]) D.row[m][(int64_t)i * D.ny[m] + j] = static_cast<float>(e[l]);
            }
    }
    if (!isfinite(chk)) atomicOr(a.status, PC_STATUS_NONFINITE);
}

template <typename T>
int ade_pass_t(pc_ctx* c, int in, int out, cudaStream_t s) {
    FieldArgs<T> a = make_field_args<T>(c, in, out);
    AdeArgs<T> ade = make_ade_args<T>(c);
    const KernelDft<T> D = kernel_dft<T>(c, 2);  // (plan_fused_dft: only with a single region)
    for (int r = 0; r < ade.nreg; ++r) {
        const int* b = ade.box[r];
        const int nxb = std::min(b[1], c->g.nx) - b[0], nyb = std::min(b[3], c->g.ny) - b[2];
        const int nzb = std::min(b[5], c->g.nz) - b[4];
        if (nxb <= 0 || nyb <= 0 || nzb <= 0) continue;
        dim3 blk(32, 8);
        bool vec = false;
        if constexpr (sizeof(T) == 4) {
            // the region's arrays and every field row are 8-byte aligned at even k - b[4]
            const int zb = b[5] - b[4];
            const bool single = ade.nreg == 1 && b[5] <= c->g.nz - 1;
            // (two points per thread: 78 registers, three CTAs per SM; four points
            // take 140 registers and one CTA per SM and run slower)
            if (single && b[4] % 2 == 0 && zb % 2 == 0) {
                ade_pass3v<T, 2><<<dim3((zb / 2 + 31) / 32, (nyb + 7) / 8, nxb), blk, 0, s>>>(a, ade, D);
                vec = true;
            }
        }
        if (!vec) ade_pass3<T><<<dim3((nzb + 31) / 32, (nyb + 7) / 8, nxb), blk, 0, s>>>(a, ade, r, D);
        ++c->launches;
    }
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

template <typename T>
int split_step_t(pc_ctx* c, cudaStream_t s, const double* tfsf_amp) {
    FieldArgs<T> a = make_field_args<T>(c, c->cur, c->cur);
    CpmlArgs<T> p = make_cpml_args<T>(c, c->cur, c->cur);
    AdeArgs<T> ade = make_ade_args<T>(c);
    const pc_grid_desc& g = c->g;
    const bool cp = p.t > 0, ad = ade.nreg > 0;
    if (g.ndim == 3) {
        dim3 blk(32, 8);
        dim3 grd((g.nz + 31) / 32, (g.ny + 7) / 8, g.nx);
        if (cp)
            split_h3<T, true><<<grd, blk, 0, s>>>(a, p);
        else
            split_h3<T, false><<<grd, blk, 0, s>>>(a, p);
        if (tfsf_amp) {
            const int rc = launch_tfsf_h(c, s);
            if (rc) return rc;
        }
        if (cp && ad)
            split_e3<T, true, true><<<grd, blk, 0, s>>>(a, p, ade);
        else if (cp)
            split_e3<T, true, false><<<grd, blk, 0, s>>>(a, p, ade);
        else if (ad)
            split_e3<T, false, true><<<grd, blk, 0, s>>>(a, p, ade);
        else
            split_e3<T, false, false><<<grd, blk, 0, s>>>(a, p, ade);
        if (tfsf_amp) {
            const int rc = launch_tfsf_e(c, *tfsf_amp, s);
            if (rc) return rc;
        }
    } else {
        dim3 blk(32, 8);
        dim3 grd((g.ny + 31) / 32, (g.nx + 7) / 8);
        if (cp)
            split_h2<T, true><<<grd, blk, 0, s>>>(a, p);
        else
            split_h2<T, false><<<grd, blk, 0, s>>>(a, p);
        if (cp && ad)
            split_e2<T, true, true><<<grd, blk, 0, s>>>(a, p, ade);
        else if (cp)
            split_e2<T, true, false><<<grd, blk, 0, s>>>(a, p, ade);
        else if (ad)
            split_e2<T, false, true><<<grd, blk, 0, s>>>(a, p, ade);
        else
            split_e2<T, false, false><<<grd, blk, 0, s>>>(a, p, ade);
    }
    c->launches += 2;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

}  // namespace

int launch_ade_pass(pc_ctx* c, int in_set, int out_set, cudaStream_t s) {
    if (c->g.ndim != 3) return PC_ERR_INVALID;
    return c->g.precision == 8 ? ade_pass_t<double>(c, in_set, out_set, s) : ade_pass_t<float>(c, in_set, out_set, s);
}

int launch_split_step(pc_ctx* c, cudaStream_t s, const double* tfsf_amp) {
    return c->g.precision == 8 ? split_step_t<double>(c, s, tfsf_amp) : split_step_t<float>(c, s, tfsf_amp);
}

}  // namespace pc
