// Device helpers shared by the corrected-stepper kernels.
#pragma once

#include "pc_internal.cuh"

namespace pc {

struct Idx3 {
    int i, j, k, nx, ny, nz, pitch;
};
struct Idx2 {
    int i, j, nx, ny, pitch;
};

template <typename T>
__device__ __forceinline__ T hcoef(const T* p, int64_t o, T s) {
    return p ? p[o] : s;
}
template <typename T>
__device__ __forceinline__ T ecoef(const T* p, int64_t o) {
    return p ? p[o] : T(1);
}

// Slab index of idx along an axis of length n with thickness t, or -1.
__device__ __forceinline__ int slab_of(int idx, int n, int t) {
    return idx < t ? idx : (idx >= n - t ? idx - (n - 2 * t) : -1);
}

// CPML-modified derivative for a 3D point: returns kinv*d + psi after
// psi <- b psi + a d.  AX selects the derivative axis (0=x, 1=y, 2=z).
template <typename T, int AX>
__device__ __forceinline__ T cpml3(const CpmlArgs<T>& p, int slot, const Idx3& q, T d) {
    const int idx = AX == 0 ? q.i : (AX == 1 ? q.j : q.k);
    const int n = AX == 0 ? q.nx : (AX == 1 ? q.ny : q.nz);
    const int s = slab_of(idx, n, p.t);
    if (s < 0) return d;
    int64_t po;
    if (AX == 0)
        po = ((int64_t)s * q.ny + q.j) * q.pitch + q.k;
    else if (AX == 1)
        po = ((int64_t)q.i * (2 * p.t) + s) * q.pitch + q.k;
    else
        po = ((int64_t)q.i * q.ny + q.j) * (2 * p.t) + s;
    po += p.axis_base[AX] + (int64_t)slot * p.slot_elems[AX];
    if ((uint64_t)po >= (uint64_t)p.total) {  // range check: flag and skip
        atomicOr(p.status, PC_STATUS_BOUNDS);
        return d;
    }
    const T psi = p.b[AX][idx] * p.psi_in[po] + p.a[AX][idx] * d;
    p.psi_out[po] = psi;
    return d * p.kinv[AX][idx] + psi;
}

template <typename T, int AX>
__device__ __forceinline__ T cpml2(const CpmlArgs<T>& p, int slot, const Idx2& q, T d) {
    const int idx = AX == 0 ? q.i : q.j;
    const int n = AX == 0 ? q.nx : q.ny;
    const int s = slab_of(idx, n, p.t);
    if (s < 0) return d;
    int64_t po;
    if (AX == 0)
        po = (int64_t)s * q.pitch + q.j;
    else
        po = (int64_t)q.i * (2 * p.t) + s;
    po += p.axis_base[AX] + (int64_t)slot * p.slot_elems[AX];
    if ((uint64_t)po >= (uint64_t)p.total) {  // range check: flag and skip
        atomicOr(p.status, PC_STATUS_BOUNDS);
        return d;
    }
    const T psi = p.b[AX][idx] * p.psi_in[po] + p.a[AX][idx] * d;
    p.psi_out[po] = psi;
    return d * p.kinv[AX][idx] + psi;
}

template <typename T>
static AdeArgs<T> make_ade_args(pc_ctx* c) {
    AdeArgs<T> A{};
    A.nreg = c->ade_n;
    A.sdt = T(c->ade_sdt);
    A.dt = T(c->g.dt);
    for (int r = 0; r < c->ade_n; ++r) {
        const pc_ade_region& R = c->ade[r];
        for (int q = 0; q < 6; ++q) A.box[r][q] = R.box[q];
        A.npoles[r] = R.npoles;
        A.ce[r] = T(c->ade_ce[r]);
        A.inv[r] = T(c->ade_inv[r]);
        for (int p = 0; p < R.npoles; ++p) {
            A.kind[r][p] = R.kind[p];
            A.c0[r][p] = T(R.c0[p]);
            A.c1[r][p] = T(R.c1[p]);
            // Lorentz: c2 carries C2 + C3 - 1 (formed in float64) for the increment form
            A.c2[r][p] = T(R.kind[p] == 0 ? (R.c2[p] + R.c3[p]) - 1.0 : R.c2[p]);
            A.c3[r][p] = T(R.c3[p]);
            for (int comp = 0; comp < 3; ++comp)
                for (int w = 0; w < 2; ++w) A.aux[r][comp][p][w] = static_cast<T*>(R.aux[comp][p][w]);
        }
    }
    return A;
}

// The dispersive region holding (i, j, k): the first region whose box contains
// it, or -1.
template <typename T>
__device__ __forceinline__ int ade_region_of(const AdeArgs<T>& A, int i, int j, int k) {
    for (int r = 0; r < A.nreg; ++r) {
        const int* b = A.box[r];
        if (i >= b[0] && i < b[1] && j >= b[2] && j < b[3] && k >= b[4] && k < b[5]) return r;
    }
    return -1;
}

// First part of the ADE E update in region r: the terms of E^n and of the
// (CPML-modified) curl.
template <typename T>
__device__ __forceinline__ T ade_partial(T ce, T inv, T sdt, T e0, T curl) {
    return ce * e0 + inv * (sdt * curl);
}

// Second part: subtract the poles' terms from the partial value, advance the
// auxiliaries of the point (offset o in the region's arrays) and return E^{n+1}.
template <typename T>
__device__ __forceinline__ T ade_poles(const AdeArgs<T>& A, int r, int comp, int64_t o, T e0, T acc) {
    for (int p = 0; p < A.npoles[r]; ++p) {
        const T a0 = A.aux[r][comp][p][0][o];
        if (A.kind[r][p] == 0) {
            // (C2 - 1) P + C3 P- = (C2 + C3 - 1) P - C3 D, with D = P - P-
            const T d1 = A.aux[r][comp][p][1][o];
            acc -= A.inv[r] * (A.c2[r][p] * a0 - A.c3[r][p] * d1);
        } else if (A.kind[r][p] == 1) {
            acc -= A.inv[r] * (T(0.5) * A.dt * (T(1) + A.c1[r][p]) * a0);
        } else {
            acc -= A.inv[r] * ((A.c1[r][p] - T(1)) * a0);
        }
    }
    const T e1 = acc;
    for (int p = 0; p < A.npoles[r]; ++p) {
        T* x0 = A.aux[r][comp][p][0];
        const T a0 = x0[o];
        if (A.kind[r][p] == 0) {
            // D+ = C0 E+ + C1 E + (C2 + C3 - 1) P - C3 D,  P+ = P + D+
            T* x1 = A.aux[r][comp][p][1];
            const T dn = (A.c0[r][p] * e1 + A.c1[r][p] * e0) + (A.c2[r][p] * a0 - A.c3[r][p] * x1[o]);
            x1[o] = dn;
            x0[o] = a0 + dn;
        } else {
            x0[o] = A.c1[r][p] * a0 + A.c0[r][p] * (T(0.5) * (e1 + e0));
        }
    }
    return e1;
}

// Offset of (i, j, k) in the auxiliary arrays of region r (box-local, k fastest).
template <typename T>
__device__ __forceinline__ int64_t ade_offset(const AdeArgs<T>& A, int r, int i, int j, int k) {
    const int* b = A.box[r];
    return ((int64_t)(i - b[0]) * (b[3] - b[2]) + (j - b[2])) * (b[5] - b[4]) + (k - b[4]);
}

// ADE update of one E component at (i, j, k) given E^n and the (CPML-modified)
// curl; returns true and E^{n+1} in e when the point lies in a dispersive region.
template <typename T>
__device__ __forceinline__ bool ade_update(const AdeArgs<T>& A, int comp, int i, int j, int k, T curl, T& e) {
    const int r = ade_region_of(A, i, j, k);
    if (r < 0) return false;
    const T e0 = e;
    e = ade_poles(A, r, comp, ade_offset(A, r, i, j, k), e0, ade_partial(A.ce[r], A.inv[r], A.sdt, e0, curl));
    return true;
}

template <typename T>
static FieldArgs<T> make_field_args(pc_ctx* c, int in_set, int out_set) {
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
        a.Ein[q] = static_cast<const T*>(c->F[in_set][q]);
        a.Hin[q] = static_cast<const T*>(c->F[in_set][3 + q]);
        a.Eout[q] = static_cast<T*>(c->F[out_set][q]);
        a.Hout[q] = static_cast<T*>(c->F[out_set][3 + q]);
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
static CpmlArgs<T> make_cpml_args(pc_ctx* c, int in_set, int out_set) {
    CpmlArgs<T> p{};
    p.t = c->cpml_t;
    if (p.t <= 0) return p;
    const pc_grid_desc& g = c->g;
    const int n[3] = {g.nx, g.ny, g.ndim == 3 ? g.nz : 0};
    const T* base = static_cast<const T*>(c->d_cpml_coef);
    int64_t off = 0;
    for (int ax = 0; ax < 3; ++ax) {
        p.b[ax] = base + off;
        p.a[ax] = base + off + n[ax];
        p.kinv[ax] = base + off + 2 * n[ax];
        off += 3 * (int64_t)n[ax];
    }
    PsiLayout L = psi_layout(g, p.t);
    for (int ax = 0; ax < 3; ++ax) {
        p.slot_elems[ax] = L.slot_elems[ax];
        p.axis_base[ax] = L.axis_base[ax];
    }
    p.total = L.total;
    p.status = c->d_status;
    p.slabc = static_cast<const T*>(c->d_cpml_slab);
    p.psi_in = static_cast<const T*>(c->psi[in_set] ? c->psi[in_set] : c->psi[0]);
    p.psi_out = static_cast<T*>(c->psi[out_set] ? c->psi[out_set] : c->psi[0]);
    return p;
}

}  // namespace pc
