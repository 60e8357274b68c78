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

int launch_split_step(pc_ctx* c, cudaStream_t s, const double* tfsf_amp) {
    return c->g.precision == 8 ? split_step_t<double>(c, s, tfsf_amp) : split_step_t<float>(c, s, tfsf_amp);
}

}  // namespace pc
