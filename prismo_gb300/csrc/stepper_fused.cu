// Corrected Yee stepper, fused schedule: one pass per time step computes
// H^{n+1/2} and E^{n+1} together (the same update rules as stepper_split.cu).
//
// Layout of the work: a CTA owns a TY x TZ tile of (j, k) and streams along x
// over a chunk of planes [ib, ie).  For each plane p it computes H^{n+1/2}(p)
// from E^n(p), E^n(p-1), then E^{n+1}(p-1) from H^{n+1/2}(p-1), H^{n+1/2}(p).
// Planes of E^n (with a one-cell halo in j and k), H^n (with a +1 halo) and Cb
// are staged in shared memory by TMA tile loads into an S-deep mbarrier ring,
// so HBM reads overlap the stencil arithmetic without register staging.
//
// Reads come from field set `cur`, writes go to set `cur^1` (ping-pong): a
// neighbouring CTA may still be reading this CTA's halo of E^n while this CTA
// writes E^{n+1}.  The CPML psi arrays ping-pong for the same reason: halo H
// points are computed redundantly but their psi is written only by the owner.
//
// Work items (tile, x-chunk) are classified by the CPML slab axes they touch;
// each class has a kernel body compiled for exactly those axes (no CPML code for
// the interior).  In float32 without per-cell H / Ca coefficients all classes
// run in one launch (fused3_multi, the class stored in the item) from a single
// longest-first queue; otherwise a plain and a general launch run on two streams.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "pc_internal.cuh"
#include "stencil_common.cuh"
#include "tma.cuh"

namespace pc {

struct FusedMaps {
    CUtensorMap e[3];
    CUtensorMap h[3];
    CUtensorMap cb[3];  // Cb of the E update, staged with the fields
};

// Work the fused kernel does for dispersive regions, a TFSF plane and plane DFT
// monitors (all zero: none).  E points inside an ADE box get the partial update
// ade_partial (the pole terms follow in ade_pass3); the TFSF plane corrections of
// tfsf.cu are added to H at k = tf_kH and to E at k = tf_k0, from the incident
// values that tfsf_line wrote for this step; the final E of a monitored plane
// point is written to its monitor's ring row (what dft_sample would copy).
template <typename T>
struct FusedXtra {
    int nbox;
    int box[PC_MAX_ADE_REGIONS][6];
    T ce[PC_MAX_ADE_REGIONS], inv[PC_MAX_ADE_REGIONS];
    T sdt;
    int tf_on, tf_kH, tf_k0, tf_pol;  // pol 0: Hy at kH and Ex at k0; 1: Hx and Ey
    T tf_sgn;
    const T* tf_inc;  // [2]: incident E at step n, incident H at n+1/2
    KernelDft<T> dft;  // plane DFT monitors sampled from the E epilogue
};

namespace {

constexpr uint32_t kWaitLimit = 1u << 22;
// plane DFT monitors the fused kernel samples (one: a second one spills registers
// of the E epilogue; further planes keep their dft_sample launch)
constexpr int kFusedDft = 1;

// Tile geometry: a CTA updates a TY x TZ tile of (j, k) for every plane of its
// x-chunk.  Eight consumer warps own the tile (lane = k, RPT rows per thread);
// a ninth helper warp issues the TMA loads and computes the 2*TZ+... halo H
// points (row j0+TY and column k0+TZ) that the E update needs.
template <typename T, int TY, int TZ>
struct FusedGeom {
    static constexpr int EW = TZ + 8;  // E box: k in [k0-4, k0+TZ+4)
    static constexpr int EH = TY + 2;  //        j in [j0-1, j0+TY+1)
    static constexpr int HW = TZ + 4;  // H box: k in [k0, k0+TZ+4)
    static constexpr int HH = TY + 1;  //        j in [j0, j0+TY+1)
    static constexpr int NW = TZ + 1;  // H^{n+1/2} smem row stride
    static constexpr int align128(int b) { return (b + 127) / 128 * 128; }
    static constexpr int E_BOX = align128(EW * EH * (int)sizeof(T));
    static constexpr int H_BOX = align128(HW * HH * (int)sizeof(T));
    static constexpr int CB_BOX = align128(TZ * TY * (int)sizeof(T));  // Cb: k in [k0, k0+TZ), j in [j0, j0+TY)
    static constexpr int STAGE = 3 * (E_BOX + H_BOX + CB_BOX);
    static constexpr uint32_t TX_BYTES = 3u * (EW * EH + HW * HH + TZ * TY) * sizeof(T);
    static constexpr int HN_PLANE = 3 * HH * NW;  // elements of one H^{n+1/2} plane (3 comps)
    static constexpr int NHALO = (TZ + 1) + TY;   // halo H points per plane
};

template <typename T, int TY, int TZ, int S>
constexpr int fused_smem_bytes() {
    using G = FusedGeom<T, TY, TZ>;
    return 256 + S * G::STAGE + 3 * G::HN_PLANE * (int)sizeof(T);
}

// One CPML recursion step: psi' = b psi + a d; returns kinv d + psi'.
template <typename T>
__device__ __forceinline__ T pstep(T b, T a, T kinv, T d, T& psi) {
    psi = b * psi + a * d;
    return d * kinv + psi;
}

// CPML state of one point: slab indices, the six psi values (slot order xA, xB,
// yA, yB, zA, zB) and the 32-bit offsets of its x, y, z psi entries (slot 0).
template <typename T>
struct PsiPoint {
    int sx, sy, sz;
    int ox, oy, oz;
};

// Work-item classes of one step: items whose planes and tile (with its +1 halo)
// touch the CPML slabs of no axis, of every axis, or of exactly the named ones.
enum { CL_PLAIN, CL_GEN, CL_YZ, CL_XZ, CL_XY, CL_Z, CL_Y, CL_X, CL_N };

// One work item of the fused step.  RPT = 2 rows per consumer thread: rows warp and
// warp + TY/2 of the tile.  AX: the CPML axes this variant handles (bit 0 x, bit 1
// y, bit 2 z; 0 = no CPML code); the host gives a variant only items whose planes
// and tile (with halo) stay clear of the slabs of the other axes.
template <typename T, int TY, int TZ, int S, int AX, bool HCOEF, bool CA, bool DFT = false>
__device__ __forceinline__ void fused3_item(const FieldArgs<T>& a, const CpmlArgs<T>& pm, const int4 item,
                                            const FusedMaps& maps, const FusedXtra<T>& xt) {
    using G = FusedGeom<T, TY, TZ>;
    constexpr bool CPML = AX != 0, CX = (AX & 1) != 0, CY = (AX & 2) != 0, CZ = (AX & 4) != 0;
    constexpr int EW = G::EW, HW = G::HW, NW = G::NW;
    constexpr int NWC = TY / 2;  // consumer warps
    static_assert(TZ == 32, "one warp spans the tile in k");
    static_assert(S >= 3, "stage n-2 is recycled while stages n-1 and n are in use");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // explicit 128-byte alignment of every TMA destination
    unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    unsigned char* stages = smem + 128;
    T* sHn = reinterpret_cast<T*>(stages + S * G::STAGE);
    T* sC = sHn + 3 * G::HN_PLANE;  // CPML slab coefficients [axis][b, a, kinv][2t]

    const int lane = threadIdx.x, warp = threadIdx.y;
    const int tid = warp * 32 + lane;
    const bool helper = warp == NWC;
    // work item: (k0, j0, first plane, one past the last plane)
    const int k0 = item.x, j0 = item.y;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int ib = item.z;
    const int ie = item.w;
    const int L = ie - ib + 2;  // planes ib-1 .. ie
    const int64_t P = a.pitch;
    const int64_t PR = (int64_t)ny * P;  // plane stride
    const int t = CPML ? pm.t : 0;
    const int t2 = 2 * t;
    const T idx_ = a.inv_dx, idy = a.inv_dy, idz = a.inv_dz;
    // dispersive regions this item's E planes [ib, ie) and tile reach; TFSF values
    // (the region loops are unrolled so that xt is indexed statically: a dynamic
    // index into a kernel parameter would copy it to local memory).  XT: the
    // variants that compile this work (not the float32 ones with per-cell H or Ca
    // coefficients, whose registers it would spill; such grids step on the split
    // kernels when they have ADE regions or a TFSF plane, fused_extras_ok).
    constexpr bool XT = sizeof(T) == 8 || (!HCOEF && !CA);
    bool ade_cta = false;
#pragma unroll
    for (int r = 0; r < PC_MAX_ADE_REGIONS; ++r) {
        const int* b = xt.box[r];
        ade_cta = ade_cta || (XT && r < xt.nbox && ib < b[1] && ie > b[0] && j0 < b[3] && j0 + TY > b[2] &&
                              k0 < b[5] && k0 + TZ > b[4]);
    }
    const bool tf_h = XT && xt.tf_on && xt.tf_kH >= k0 && xt.tf_kH <= k0 + TZ;  // incl. the helper's halo column
    const bool tf_e = XT && xt.tf_on && xt.tf_k0 >= k0 && xt.tf_k0 < k0 + TZ;
    const T inc_h = tf_h ? xt.tf_inc[0] : T(0);
    const T inc_e = tf_e ? xt.tf_inc[1] : T(0);
    bool dft_cta = false;  // a monitored plane crosses this tile (DFT: the instantiation that samples)
    if (DFT) {
#pragma unroll
        for (int m = 0; m < kFusedDft; ++m)
            dft_cta = dft_cta || (m < xt.dft.n && xt.dft.k[m] >= k0 && xt.dft.k[m] < k0 + TZ);
    }

    if (helper && lane == 0) {
        for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
        for (int c = 0; c < 3; ++c) {
            prefetch_tmap(&maps.e[c]);
            prefetch_tmap(&maps.h[c]);
        }
    }
    if (CPML)
        for (int i = tid; i < 9 * t2; i += blockDim.x * blockDim.y) sC[i] = pm.slabc[i];
    __syncthreads();

    auto issue = [&](int n) {
        const int s = n % S;
        unsigned char* st = stages + s * G::STAGE;
        const int pl = ib - 1 + n;
        mbar_expect_tx(&bars[s], G::TX_BYTES);
#pragma unroll
        for (int c = 0; c < 3; ++c) tma_load_3d(st + c * G::E_BOX, &maps.e[c], k0 - 4, j0 - 1, pl, &bars[s]);
#pragma unroll
        for (int c = 0; c < 3; ++c)
            tma_load_3d(st + 3 * G::E_BOX + c * G::H_BOX, &maps.h[c], k0, j0, pl, &bars[s]);
#pragma unroll
        for (int c = 0; c < 3; ++c)
            tma_load_3d(st + 3 * (G::E_BOX + G::H_BOX) + c * G::CB_BOX, &maps.cb[c], k0, j0, pl, &bars[s]);
    };
    int issued = L < S ? L : S;
    if (helper && lane == 0)
        for (int n = 0; n < issued; ++n) issue(n);

    // ---- CPML bookkeeping (32-bit offsets: the host guarantees psi < 2^31 elements) ----
    const int P32 = (int)P;
    const int se0 = (int)pm.slot_elems[0], se1 = (int)pm.slot_elems[1], se2 = (int)pm.slot_elems[2];
    const int tot = (int)pm.total;
    auto sl_of = [&](int i, int nn) { return (CPML && i >= 0 && i < nn) ? slab_of(i, nn, t) : -1; };
    // coefficient triplet (b, a, kinv) of slab index sl on axis ax (1, 0, 1 outside)
    auto coef3 = [&](int ax, int sl, T& b, T& aa, T& kk) {
        if (sl >= 0) {
            b = sC[(ax * 3 + 0) * t2 + sl];
            aa = sC[(ax * 3 + 1) * t2 + sl];
            kk = sC[(ax * 3 + 2) * t2 + sl];
        } else {
            b = T(1), aa = T(0), kk = T(1);
        }
    };
    // psi accesses: range-checked once per work item (psi_ok, below) instead of per
    // access; a thread whose offsets could leave [0, tot) flags PC_STATUS_BOUNDS and
    // skips its psi traffic
    bool psi_ok = true;
    auto ld = [&](int o) -> T { return psi_ok ? __ldg(pm.psi_in + o) : T(0); };
    auto st = [&](int o, T v) {
        if (psi_ok) pm.psi_out[o] = v;
    };
    // point state for plane pl of a point (j, k) with per-point constants
    // (syc, szc: slab indices; oyc/ozc: plane-independent parts of the offsets)
    auto make_pt = [&](int pl, int sxp, int syc, int szc, int oxc, int oyc, int ozc) {
        PsiPoint<T> q;
        const bool pv = pl >= 0 && pl < nx;
        q.sx = pv ? sxp : -1;
        q.sy = pv ? syc : -1;
        q.sz = pv ? szc : -1;
        q.ox = oxc + (q.sx >= 0 ? q.sx : 0) * (ny * P32);
        q.oy = oyc + pl * (t2 * P32);
        q.oz = ozc + pl * (ny * t2);
        return q;
    };
    // slot offsets of H and E psi entries inside an axis block
    const int xA_H = SX_HY * se0, xB_H = SX_HZ * se0, yA_H = SY_HX * se1, yB_H = SY_HZ * se1;
    const int zA_H = SZ_HX * se2, zB_H = SZ_HY * se2;
    const int xA_E = SX_EY * se0, xB_E = SX_EZ * se0, yA_E = SY_EX * se1, yB_E = SY_EZ * se1;
    const int zA_E = SZ_EX * se2, zB_E = SZ_EY * se2;
    auto fetch = [&](const PsiPoint<T>& q, bool isH, T* v) {
#pragma unroll
        for (int w = 0; w < 6; ++w) v[w] = T(0);
        if (CX && q.sx >= 0) {
            v[0] = ld(q.ox + (isH ? xA_H : xA_E));
            v[1] = ld(q.ox + (isH ? xB_H : xB_E));
        }
        if (CY && q.sy >= 0) {
            v[2] = ld(q.oy + (isH ? yA_H : yA_E));
            v[3] = ld(q.oy + (isH ? yB_H : yB_E));
        }
        if (CZ && q.sz >= 0) {
            v[4] = ld(q.oz + (isH ? zA_H : zA_E));
            v[5] = ld(q.oz + (isH ? zB_H : zB_E));
        }
    };

    // ---- per-thread points -------------------------------------------------
    // Consumers own rows (warp, warp + TY/2) at lane k; the helper owns the two halo
    // points h = lane, lane + 32 (row j0+TY, then column k0+TZ).  Same registers.
    int pj[2], pk[2], pei[2], pho[2], pno[2], psy[2], psz[2], poxc[2], poyc[2], pozc[2];
    bool pin[2];  // point exists and lies inside the domain
    T pyb[2], pya[2], pyk[2], pzb[2], pza[2], pzk[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        int jj, kk;
        bool exists = true;
        if (!helper) {
            jj = warp + NWC * r;
            kk = lane;
        } else {
            const int h = lane + 32 * r;
            exists = h < G::NHALO;
            jj = h <= TZ ? TY : h - (TZ + 1);
            kk = h <= TZ ? h : TZ;
        }
        pj[r] = j0 + jj;
        pk[r] = k0 + kk;
        pei[r] = (jj + 1) * EW + (kk + 4);
        pho[r] = jj * HW + kk;
        pno[r] = jj * NW + kk;
        pin[r] = exists && pj[r] < ny && pk[r] < nz;
        psy[r] = (CY && pin[r]) ? sl_of(pj[r], ny) : -1;
        psz[r] = (CZ && pin[r]) ? sl_of(pk[r], nz) : -1;
        coef3(1, psy[r], pyb[r], pya[r], pyk[r]);
        coef3(2, psz[r], pzb[r], pza[r], pzk[r]);
        poxc[r] = (int)pm.axis_base[0] + pj[r] * P32 + pk[r];
        poyc[r] = (int)pm.axis_base[1] + (psy[r] >= 0 ? psy[r] : 0) * P32 + pk[r];
        pozc[r] = (int)pm.axis_base[2] + pj[r] * t2 + (psz[r] >= 0 ? psz[r] : 0);
    }
    // dispersive regions holding each of the thread's (j, k) points (bit per region)
    unsigned ade_jk[2] = {0u, 0u};
    if (ade_cta) {
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int rr = 0; rr < PC_MAX_ADE_REGIONS; ++rr) {
                const int* b = xt.box[rr];
                if (rr < xt.nbox && pj[r] >= b[2] && pj[r] < b[3] && pk[r] >= b[4] && pk[r] < b[5])
                    ade_jk[r] |= 1u << rr;
            }
    }
    if (CPML) {
        // every offset a point can form over this item's planes: x-slab entries at any
        // slab index, y/z-slab entries up to the last plane, plus the largest slot
        const int64_t sxm = max(max(xA_H, xB_H), max(xA_E, xB_E));
        const int64_t sym = max(max(yA_H, yB_H), max(yA_E, yB_E));
        const int64_t szm = max(max(zA_H, zB_H), max(zA_E, zB_E));
        const int64_t phi = min(ie, nx - 1);
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            if (!pin[r]) continue;
            const int64_t lo_x = poxc[r], hi_x = (int64_t)poxc[r] + (int64_t)(t2 - 1) * ny * P32 + sxm;
            bool ok = !CX || (lo_x >= 0 && hi_x < tot);
            if (psy[r] >= 0) ok = ok && poyc[r] >= 0 && (int64_t)poyc[r] + phi * t2 * P32 + sym < tot;
            if (psz[r] >= 0) ok = ok && pozc[r] >= 0 && (int64_t)pozc[r] + phi * ny * t2 + szm < tot;
            psi_ok = psi_ok && ok;
        }
        if (!psi_ok) atomicOr(pm.status, PC_STATUS_BOUNDS);
    }
    const int k = k0 + lane;  // consumers' own k
    auto pt_at = [&](int pl, int r) {
        return make_pt(pl, (CX && pin[r]) ? sl_of(pl, nx) : -1, psy[r], psz[r], poxc[r], poyc[r], pozc[r]);
    };
    auto og = [&](int pl, int r) { return (int64_t)pl * PR + (int64_t)pj[r] * P + pk[r]; };
    // CTA-uniform: does the tile touch a y or z slab (then every plane needs CPML)?
    // (the +1 halo row/column of H counts: E at the tile edge reads it)
    const bool yz_slab = (CY && (j0 < t || j0 + TY >= ny - t)) || (CZ && (k0 < t || k0 + TZ >= nz - t));
    auto x_slab = [&](int pl) { return CX && pl >= 0 && pl < nx && (pl < t || pl >= nx - t); };

    // ---- H^{n+1/2} at one point --------------------------------------------
    auto h_compute = [&](const T* E0, const T* E1, const T* E2, const T* Ep1, const T* Ep2, const T* H0,
                         const T* H1, const T* H2, int ei, int ho, int p, int j, int kk, bool own, bool slab,
                         const PsiPoint<T>& q, T xb, T xa, T xk, T b1, T a1, T k1, T b2, T a2, T k2, T* v,
                         int64_t og, T& hx, T& hy, T& hz) {
        const bool pin = p >= 1 && p <= nx - 2;
        const bool jin = j >= 1 && j <= ny - 2;
        const bool kin = kk >= 1 && kk <= nz - 2;
        const bool ux = p >= 0 && p <= nx - 2 && jin && kin;
        const bool uy = pin && j <= ny - 2 && kin;
        const bool uz = pin && jin && kk <= nz - 2;
        const T ez = E2[ei], ey = E1[ei], ex = E0[ei];
        // derivatives in psi slot order: (dEz/dx Hy, dEy/dx Hz, dEz/dy Hx, dEx/dy Hz, dEy/dz Hx, dEx/dz Hy)
        T d0 = (ez - Ep2[ei]) * idx_;
        T d1 = (ey - Ep1[ei]) * idx_;
        T d2 = (ez - E2[ei - EW]) * idy;
        T d3 = (ex - E0[ei - EW]) * idy;
        T d4 = (ey - E1[ei - 1]) * idz;
        T d5 = (ex - E0[ei - 1]) * idz;
        if (CPML && slab) {
            if (CX && q.sx >= 0) {
                d0 = pstep(xb, xa, xk, d0, v[0]);
                d1 = pstep(xb, xa, xk, d1, v[1]);
                if (own && uy) st(q.ox + xA_H, v[0]);
                if (own && uz) st(q.ox + xB_H, v[1]);
            }
            if (CY && q.sy >= 0) {
                d2 = pstep(b1, a1, k1, d2, v[2]);
                d3 = pstep(b1, a1, k1, d3, v[3]);
                if (own && ux) st(q.oy + yA_H, v[2]);
                if (own && uz) st(q.oy + yB_H, v[3]);
            }
            if (CZ && q.sz >= 0) {
                d4 = pstep(b2, a2, k2, d4, v[4]);
                d5 = pstep(b2, a2, k2, d5, v[5]);
                if (own && ux) st(q.oz + zA_H, v[4]);
                if (own && uy) st(q.oz + zB_H, v[5]);
            }
        }
        hx = H0[ho];
        hy = H1[ho];
        hz = H2[ho];
        T da0 = a.da_s, da1 = a.da_s, da2 = a.da_s, db0 = a.db_s, db1 = a.db_s, db2 = a.db_s;
        if (HCOEF) {
            if (ux) da0 = a.da[0][og], db0 = a.db[0][og];
            if (uy) da1 = a.da[1][og], db1 = a.db[1][og];
            if (uz) da2 = a.da[2][og], db2 = a.db[2][og];
        }
        if (ux) hx = da0 * hx - db0 * (d2 - d4);
        if (uy) hy = da1 * hy - db1 * (d5 - d0);
        if (uz) hz = da2 * hz - db2 * (d1 - d3);
        if (tf_h && kk == xt.tf_kH) {  // TFSF plane correction (tfsf_h's ranges: the update ranges here)
            if (xt.tf_pol == 0) {
                if (uy) hy += xt.tf_sgn * db1 * inc_h * idz;
            } else {
                if (ux) hx += xt.tf_sgn * db0 * inc_h * idz;
            }
        }
    };

    bool timed_out = false;
    int n = 0;
    int sn = 0, sp = S - 1;  // stage of plane n and n-1
    int hc = 0, hp = 2;      // H^{n+1/2} smem buffer of plane n and n-1
    T pfH[2][6], pfE[2][6];  // psi prefetched one plane ahead (slab planes only)
    if (CPML && (yz_slab || x_slab(ib))) {
#pragma unroll
        for (int r = 0; r < 2; ++r) fetch(pt_at(ib, r), true, pfH[r]);
    }
    T chk = T(0);  // running sum of E^{n+1}: non-finite iff some value was
    for (; n < L; ++n) {
        const int p = ib - 1 + n;  // plane whose H^{n+1/2} is computed now
        const int q = p - 1;       // plane whose E^{n+1} is computed now
        const bool slabH = yz_slab || x_slab(p);
        const bool slabE = yz_slab || x_slab(q);
        const unsigned char* stc = stages + sn * G::STAGE;
        const unsigned char* stp = stages + sp * G::STAGE;
        const T* Ec0 = reinterpret_cast<const T*>(stc);
        const T* Ec1 = reinterpret_cast<const T*>(stc + G::E_BOX);
        const T* Ec2 = reinterpret_cast<const T*>(stc + 2 * G::E_BOX);
        const T* Hc0 = reinterpret_cast<const T*>(stc + 3 * G::E_BOX);
        const T* Hc1 = reinterpret_cast<const T*>(stc + 3 * G::E_BOX + G::H_BOX);
        const T* Hc2 = reinterpret_cast<const T*>(stc + 3 * G::E_BOX + 2 * G::H_BOX);
        const T* Ep0 = reinterpret_cast<const T*>(stp);
        const T* Ep1 = reinterpret_cast<const T*>(stp + G::E_BOX);
        const T* Ep2 = reinterpret_cast<const T*>(stp + 2 * G::E_BOX);
        T* Nc0 = sHn + hc * G::HN_PLANE;
        T* Nc1 = Nc0 + G::HH * NW;
        T* Nc2 = Nc1 + G::HH * NW;
        const T* Np0 = sHn + hp * G::HN_PLANE;
        const T* Np1 = Np0 + G::HH * NW;
        const T* Np2 = Np1 + G::HH * NW;
        // Cb(q) of the E update: staged by TMA with plane q's fields
        const T* Cq = reinterpret_cast<const T*>(stp + 3 * (G::E_BOX + G::H_BOX));
        // x-slab coefficients of planes p and q (uniform)
        T xbH = T(1), xaH = T(0), xkH = T(1), xbE = T(1), xaE = T(0), xkE = T(1);
        if (CX) {
            coef3(0, sl_of(p, nx), xbH, xaH, xkH);
            coef3(0, sl_of(q, nx), xbE, xaE, xkE);
        }
        const bool ok = mbar_wait_bounded(&bars[sn], (uint32_t)((n / S) & 1), kWaitLimit);
        T hv[2][3];
        if (n >= 1 && ok) {
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                if (helper && lane + 32 * r >= G::NHALO) continue;
                const PsiPoint<T> pt = pt_at(p, r);
                h_compute(Ec0, Ec1, Ec2, Ep1, Ep2, Hc0, Hc1, Hc2, pei[r], pho[r], p, pj[r], pk[r],
                          !helper && p < ie, slabH, pt, xbH, xaH, xkH, pyb[r], pya[r], pyk[r], pzb[r], pza[r],
                          pzk[r], pfH[r], og(p, r), hv[r][0], hv[r][1], hv[r][2]);
                Nc0[pno[r]] = hv[r][0];
                Nc1[pno[r]] = hv[r][1];
                Nc2[pno[r]] = hv[r][2];
            }
        }
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        if (n >= 2 && n - 2 + S < L) {
            if (helper && lane == 0) issue(n - 2 + S);
            ++issued;
        }
        // H-phase psi of the next plane: issued now so the loads overlap the E phase
        if (CPML && (yz_slab || x_slab(p + 1))) {
#pragma unroll
            for (int r = 0; r < 2; ++r) fetch(pt_at(p + 1, r), true, pfH[r]);
        }
        if (!helper) {
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int j = pj[r];
                if (!pin[r]) continue;
                if (n >= 2) {
                    const int no = pno[r];
                    const bool ux = j <= ny - 2 && k <= nz - 2;
                    const bool uy = q <= nx - 2 && k <= nz - 2;
                    const bool uz = q <= nx - 2 && j <= ny - 2;
                    const T hxq = Np0[no], hyq = Np1[no], hzq = Np2[no];
                    // derivatives in psi slot order:
                    // (dHz/dx Ey, dHy/dx Ez, dHz/dy Ex, dHx/dy Ez, dHy/dz Ex, dHx/dz Ey)
                    T d0 = (Nc2[no] - hzq) * idx_;
                    T d1 = (Nc1[no] - hyq) * idx_;
                    T d2 = (Np2[no + NW] - hzq) * idy;
                    T d3 = (Np0[no + NW] - hxq) * idy;
                    T d4 = (Np1[no + 1] - hyq) * idz;
                    T d5 = (Np0[no + 1] - hxq) * idz;
                    if (CPML && slabE) {
                        const PsiPoint<T> pt = pt_at(q, r);
                        T* v = pfE[r];
                        if (CX && pt.sx >= 0) {
                            d0 = pstep(xbE, xaE, xkE, d0, v[0]);
                            d1 = pstep(xbE, xaE, xkE, d1, v[1]);
                            if (uy) st(pt.ox + xA_E, v[0]);
                            if (uz) st(pt.ox + xB_E, v[1]);
                        }
                        if (CY && pt.sy >= 0) {
                            d2 = pstep(pyb[r], pya[r], pyk[r], d2, v[2]);
                            d3 = pstep(pyb[r], pya[r], pyk[r], d3, v[3]);
                            if (ux) st(pt.oy + yA_E, v[2]);
                            if (uz) st(pt.oy + yB_E, v[3]);
                        }
                        if (CZ && pt.sz >= 0) {
                            d4 = pstep(pzb[r], pza[r], pzk[r], d4, v[4]);
                            d5 = pstep(pzb[r], pza[r], pzk[r], d5, v[5]);
                            if (ux) st(pt.oz + zA_E, v[4]);
                            if (uy) st(pt.oz + zB_E, v[5]);
                        }
                    }
                    const int ei = pei[r];
                    T ex = Ep0[ei], ey = Ep1[ei], ez = Ep2[ei];
                    const int64_t o = og(q, r);
                    T ca0 = T(1), ca1 = T(1), ca2 = T(1);
                    if (CA) {
                        ca0 = a.ca[0][o];
                        ca1 = a.ca[1][o];
                        ca2 = a.ca[2][o];
                    }
                    const int cbo = (warp + NWC * r) * TZ + lane;
                    const T cb0 = Cq[cbo], cb1 = Cq[G::CB_BOX / sizeof(T) + cbo], cb2 = Cq[2 * (G::CB_BOX / sizeof(T)) + cbo];
                    unsigned am = 0u;  // dispersive regions holding the point
                    if (ade_cta) {
#pragma unroll
                        for (int rr = 0; rr < PC_MAX_ADE_REGIONS; ++rr)
                            if (q >= xt.box[rr][0] && q < xt.box[rr][1]) am |= 1u << rr;
                        am &= ade_jk[r];
                    }
                    if (am) {  // partial ADE update in the first region; ade_pass3 adds the pole terms
                        T ce = T(0), iv = T(0);
#pragma unroll
                        for (int rr = PC_MAX_ADE_REGIONS - 1; rr >= 0; --rr)
                            if (am & (1u << rr)) ce = xt.ce[rr], iv = xt.inv[rr];
                        const T sdt = xt.sdt;
                        if (ux) ex = ade_partial(ce, iv, sdt, ex, d2 - d4);
                        if (uy) ey = ade_partial(ce, iv, sdt, ey, d5 - d0);
                        if (uz) ez = ade_partial(ce, iv, sdt, ez, d1 - d3);
                    } else {
                        if (ux) ex = ca0 * ex + cb0 * (d2 - d4);
                        if (uy) ey = ca1 * ey + cb1 * (d5 - d0);
                        if (uz) ez = ca2 * ez + cb2 * (d1 - d3);
                    }
                    if (tf_e && k == xt.tf_k0) {  // TFSF plane correction (tfsf_e's ranges)
                        if (xt.tf_pol == 0) {
                            if (j <= ny - 2) ex += cb0 * inc_e * idz;
                        } else {
                            if (q <= nx - 2) ey += cb1 * inc_e * idz;
                        }
                    }
                    if (DFT && dft_cta) {
#pragma unroll
                        for (int m = 0; m < kFusedDft; ++m)
                            if (m < xt.dft.n && k == xt.dft.k[m] && q < xt.dft.nx[m] && j < xt.dft.ny[m]) {
                                const T v = xt.dft.comp[m] == 0 ? ex : (xt.dft.comp[m] == 1 ? ey : ez);
                                xt.dft.row[m][(int64_t)q * xt.dft.ny[m] + j] = static_cast<float>(v);
                            }
                    }
                    a.Eout[0][o] = ex;
                    a.Eout[1][o] = ey;
                    a.Eout[2][o] = ez;
                    chk += (ex + ey) + ez;
                }
                if (n >= 1 && p < ie) {
                    const int64_t o = og(p, r);
                    a.Hout[0][o] = hv[r][0];
                    a.Hout[1][o] = hv[r][1];
                    a.Hout[2][o] = hv[r][2];
                }
            }
            if (CPML && n >= 1 && (yz_slab || x_slab(p))) {  // E-phase psi of the next iteration
#pragma unroll
                for (int r = 0; r < 2; ++r) fetch(pt_at(p, r), false, pfE[r]);
            }
        }
        sp = sn;
        sn = (sn + 1 == S) ? 0 : sn + 1;
        hp = hc;
        hc = (hc + 1 == 3) ? 0 : hc + 1;
    }
    if (!helper && !isfinite(chk)) atomicOr(a.status, PC_STATUS_NONFINITE);
    if (timed_out) {
        if (helper && lane == 0) atomicOr(a.status, PC_STATUS_TIMEOUT);
        // let every copy already in flight land before the CTA retires
        for (int m = n; m < issued; ++m) mbar_wait_bounded(&bars[m % S], (uint32_t)((m / S) & 1), kWaitLimit);
    }
}

// one kernel variant: items[blockIdx.x], longest first
template <typename T, int TY, int TZ, int S, int AX, bool HCOEF, bool CA>
__global__ void __launch_bounds__(TZ*(TY / 2 + 1), (sizeof(T) == 4 ? 2 : 1))
    fused3(FieldArgs<T> a, CpmlArgs<T> pm, const int4* __restrict__ items, const __grid_constant__ FusedMaps maps,
           const FusedXtra<T> xt) {
    fused3_item<T, TY, TZ, S, AX, HCOEF, CA>(a, pm, items[blockIdx.x], maps, xt);
}

// Every class in one launch (float32, no per-cell H or Ca coefficients): the class
// of an item sits in the top byte of its w; the CTA runs that class's variant.
// DFT: the instantiation that writes plane DFT samples from the E epilogue (only
// launched when a monitor is sampled here, so the common one keeps its registers).
template <typename T, int TY, int TZ, int S, bool DFT>
__global__ void __launch_bounds__(TZ*(TY / 2 + 1), (sizeof(T) == 4 ? 2 : 1))
    fused3_multi(FieldArgs<T> a, CpmlArgs<T> pm, const int4* __restrict__ items,
                 const __grid_constant__ FusedMaps maps, const FusedXtra<T> xt) {
    int4 it = items[blockIdx.x];
    const int cls = it.w >> 24;
    it.w &= 0xFFFFFF;
    switch (cls) {
        case CL_PLAIN: fused3_item<T, TY, TZ, S, 0, false, false, DFT>(a, pm, it, maps, xt); break;
        case CL_Z: fused3_item<T, TY, TZ, S, 4, false, false, DFT>(a, pm, it, maps, xt); break;
        case CL_Y: fused3_item<T, TY, TZ, S, 2, false, false, DFT>(a, pm, it, maps, xt); break;
        case CL_X: fused3_item<T, TY, TZ, S, 1, false, false, DFT>(a, pm, it, maps, xt); break;
        case CL_YZ: fused3_item<T, TY, TZ, S, 6, false, false, DFT>(a, pm, it, maps, xt); break;
        case CL_XZ: fused3_item<T, TY, TZ, S, 5, false, false, DFT>(a, pm, it, maps, xt); break;
        case CL_XY: fused3_item<T, TY, TZ, S, 3, false, false, DFT>(a, pm, it, maps, xt); break;
        default: fused3_item<T, TY, TZ, S, 7, false, false, DFT>(a, pm, it, maps, xt); break;
    }
}

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn get_encode() {
    static EncodeFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    }
    return fn;
}

}  // namespace

// A 3D tiled tensor map over one padded field array (k fastest, then j, then i)
// with a box of bw x bh x 1 elements; loads outside the array fill zero.
int make_map(CUtensorMap* m, const void* base, const pc_grid_desc& g, int bw, int bh) {
    EncodeFn enc = get_encode();
    if (!enc) return PC_ERR_CUDA;
    const int es = g.precision;
    cuuint64_t dims[3] = {(cuuint64_t)g.nz, (cuuint64_t)g.ny, (cuuint64_t)g.nx};
    cuuint64_t strides[2] = {(cuuint64_t)g.pitch * es, (cuuint64_t)g.ny * g.pitch * es};
    cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(m, es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                     const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? PC_OK : PC_ERR_CUDA;
}

namespace {

struct FusedState {
    const void* key_f[2][6];
    const void* key_cb[3];
    FusedMaps maps[2];  // per input set
    bool ready = false;
    int4* d_items = nullptr;  // work items of the current chunking, class after class
    int n_cls[CL_N] = {}, off_cls[CL_N] = {};
    int items_cx = -1, items_cxe = -1, items_t = -1, items_split = -1, items_unified = -1;
    // the CPML classes run here, concurrently with the plain class and each other
    cudaStream_t side[CL_N - 1] = {};
    cudaEvent_t fork = nullptr, join[CL_N - 1] = {};
};

// One cached set of maps per context (keyed by the buffer pointers).
FusedState* state_of(pc_ctx* c) {
    if (!c->fused_state) c->fused_state = new FusedState();
    return static_cast<FusedState*>(c->fused_state);
}

// Work items (k0, j0, ib, ie) for a chunk length cx, most expensive first
// (longest-processing-time-first ordering against the tail).  With a CPML an item
// touches the slabs of a set of axes: x when its planes [ib, ie] (ie = halo plane)
// reach an x slab, y / z when its tile with the +1 halo row / column reaches a y /
// z slab.  Items that touch none run the variant without CPML code (CL_PLAIN);
// with split >= 1, items that touch one axis run that axis's variant (CL_X, CL_Y,
// CL_Z: the x-chunks [0, t) and [nx-t-1, nx) of inner tiles, the edge tiles of the
// inner planes), with split 2 also items that touch two (CL_XY, CL_XZ: the end
// chunks of edge tiles; CL_YZ: the corner tiles of the inner planes); the rest run
// the general variant (CL_GEN).
// relative cost of one tile-plane per class (warp instructions per tile-plane at
// 256^3 over the plain class's): orders the items longest first
constexpr double kClassCost[CL_N] = {1.0, 3.1, 2.6, 2.6, 2.6, 1.8, 1.7, 2.0};

using CostItem = std::pair<double, int4>;

// longest first; equal costs by chunk, then tile, so that neighbouring tiles of one
// chunk run together and share their halo rows in L2
static void sort_items(std::vector<CostItem>& v) {
    std::sort(v.begin(), v.end(), [](const CostItem& x, const CostItem& y) {
        if (x.first != y.first) return x.first > y.first;
        if (x.second.z != y.second.z) return x.second.z < y.second.z;
        if (x.second.y != y.second.y) return x.second.y < y.second.y;
        return x.second.x < y.second.x;
    });
}

static void fused_items(const pc_grid_desc& g, int TY, int TZ, int cx, int cx_edge, int t, int split,
                        std::vector<CostItem> (&v)[CL_N]) {
    auto chunking = [&](int c) {
        std::vector<std::pair<int, int>> chunks;
        if (t > 0 && g.nx > 2 * t + 2) {
            chunks.push_back({0, t});
            for (int ib = t; ib < g.nx - t - 1; ib += c) chunks.push_back({ib, std::min(g.nx - t - 1, ib + c)});
            chunks.push_back({g.nx - t - 1, g.nx});
        } else {
            for (int ib = 0; ib < g.nx; ib += c) chunks.push_back({ib, std::min(g.nx, ib + c)});
        }
        return chunks;
    };
    const std::vector<std::pair<int, int>> inner = chunking(cx), edge = chunking(cx_edge);
    for (int c = 0; c < CL_N; ++c) v[c].clear();
    for (int j0 = 0; j0 < g.ny; j0 += TY)
        for (int k0 = 0; k0 < g.nz; k0 += TZ) {
            const bool ys = t > 0 && (j0 < t || j0 + TY >= g.ny - t);
            const bool zs = t > 0 && (k0 < t || k0 + TZ >= g.nz - t);
            for (auto& ch : (ys || zs) ? edge : inner) {
                const int ib = ch.first, ie = ch.second;
                const bool xs = t > 0 && (ib < t || ie >= g.nx - t);
                const int mask = (xs ? 1 : 0) | (ys ? 2 : 0) | (zs ? 4 : 0);
                static constexpr int by_mask[8] = {CL_PLAIN, CL_X, CL_Y, CL_XY, CL_Z, CL_XZ, CL_YZ, CL_GEN};
                static constexpr int axes[8] = {0, 1, 1, 2, 1, 2, 2, 3};
                const int c = (mask == 0 || axes[mask] <= split) ? by_mask[mask] : CL_GEN;
                v[c].push_back({kClassCost[c] * (ie - ib + 2), make_int4(k0, j0, ib, ie)});
            }
        }
    for (int c = 0; c < CL_N; ++c) sort_items(v[c]);
}

template <typename T, int TY, int TZ, int S, int AX, bool HCOEF, bool CA>
int launch_variant(cudaStream_t s, const FieldArgs<T>& a, const CpmlArgs<T>& p, const FusedMaps& maps,
                   const FusedXtra<T>& xt, int smem, const int4* items, int n_items) {
    auto kern = fused3<T, TY, TZ, S, AX, HCOEF, CA>;
    static bool attr = false;
    if (!attr) {  // the largest size any launch asks for (CPML table for PC_MAX_CPML)
        const int smem_max = fused_smem_bytes<T, TY, TZ, S>() + 9 * 2 * PC_MAX_CPML * (int)sizeof(T);
        PC_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
        attr = true;
    }
    if (n_items <= 0) return PC_OK;
    dim3 blk(TZ, TY / 2 + 1);
    kern<<<n_items, blk, smem, s>>>(a, p, items, maps, xt);
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

// chunk length along x: enough work items for ~8 per resident CTA slot
template <typename T, int TY, int TZ, int S>
int choose_chunk(const pc_grid_desc& g, int smem) {
    auto kern = fused3<T, TY, TZ, S, 7, false, false>;
    constexpr int threads = TZ * (TY / 2 + 1);
    int sms = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         fused_smem_bytes<T, TY, TZ, S>() + 9 * 2 * PC_MAX_CPML * (int)sizeof(T));
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (per_sm <= 0) per_sm = 1;
    const int resident = sms * per_sm;
    const int tiles = ((g.nz + TZ - 1) / TZ) * ((g.ny + TY - 1) / TY);
    int cx = g.nx;
    const int cands[] = {16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512};
    for (int cand : cands) {
        if (cand >= g.nx) break;
        const double items = (double)tiles * ((g.nx + cand - 1) / cand);
        if (items >= 8.0 * resident) cx = cand;
    }
    if (cx == g.nx) {
        for (int cand : cands)
            if (cand < g.nx && (double)tiles * ((g.nx + cand - 1) / cand) >= 2.0 * resident) cx = cand;
    }
    return cx;
}

}  // namespace

// fused_t runs every item class in one fused3_multi launch (the one launch that
// can sample DFT planes): float32, no per-cell H or Ca coefficients, CPML
static bool fused_unified_path(const pc_ctx* c) {
    return c->g.precision == 4 && !c->ca[0] && !c->da[0] && c->fused_split > 0 && c->fused_unified != 0 &&
           c->cpml_t > 0;
}

void plan_fused_dft(pc_ctx* c) {
    int n[3] = {0, 0, 0};
    const pc_grid_desc& g = c->g;
    const bool unified = fused_unified_path(c);
    for (auto& m : c->dfts) {
        m.fused = false;
        m.fused_where = 0;
        if (m.plane_k < 0 || m.comp > 2 || !c->sources.empty() || g.ndim != 3) continue;
        const int k = m.plane_k;
        bool in_box = false;
        for (int r = 0; r < c->ade_n; ++r) in_box = in_box || (k >= c->ade[r].box[4] && k < c->ade[r].box[5]);
        int where = 0;
        if (!in_box) {
            where = unified ? 1 : 0;
        } else if (c->ade_n == 1) {
            // the whole plane inside the box and inside the component's update range
            const int* b = c->ade[0].box;
            const bool inside = b[0] <= 0 && m.plane_nx <= b[1] && b[2] <= 0 && m.plane_ny <= b[3];
            const bool upd = m.comp == 0   ? (m.plane_ny <= g.ny - 1 && k <= g.nz - 2)
                             : m.comp == 1 ? (m.plane_nx <= g.nx - 1 && k <= g.nz - 2)
                                           : (m.plane_nx <= g.nx - 1 && m.plane_ny <= g.ny - 1);
            if (inside && upd) where = 2;
        }
        if (where && n[where] < (where == 1 ? kFusedDft : PC_MAX_FUSED_DFT)) {
            ++n[where];
            m.fused = true;
            m.fused_where = where;
        }
    }
}

template <typename T>
KernelDft<T> kernel_dft(const pc_ctx* c, int where) {
    KernelDft<T> d{};
    for (const auto& m : c->dfts) {
        if (!m.fused || m.fused_where != where || d.n >= PC_MAX_FUSED_DFT) continue;
        d.comp[d.n] = m.comp;
        d.k[d.n] = m.plane_k;
        d.nx[d.n] = m.plane_nx;
        d.ny[d.n] = m.plane_ny;
        d.row[d.n] = m.d_ring + (size_t)m.rows * m.npts;
        ++d.n;
    }
    return d;
}
template KernelDft<float> kernel_dft<float>(const pc_ctx*, int);
template KernelDft<double> kernel_dft<double>(const pc_ctx*, int);

namespace {

template <typename T>
FusedXtra<T> make_fused_xtra(const pc_ctx* c, bool tfsf) {
    FusedXtra<T> x{};
    x.dft = kernel_dft<T>(c, 1);
    x.nbox = c->ade_n;
    for (int r = 0; r < c->ade_n; ++r) {
        for (int q = 0; q < 6; ++q) x.box[r][q] = c->ade[r].box[q];
        x.ce[r] = T(c->ade_ce[r]);
        x.inv[r] = T(c->ade_inv[r]);
    }
    x.sdt = T(c->ade_sdt);
    if (tfsf && c->tfsf.on) {
        const TfsfState& t = c->tfsf;
        x.tf_on = 1;
        x.tf_pol = t.pol;
        x.tf_k0 = t.k0;
        x.tf_kH = t.dir > 0 ? t.k0 : t.k0 + 1;  // as in tfsf_h
        x.tf_sgn = T(((t.pol == 0) == (t.dir > 0)) ? 1 : -1);
        x.tf_inc = static_cast<const T*>(t.d_inc);
    }
    return x;
}

template <typename T, int TY, int TZ, int S>
int fused_t(pc_ctx* c, cudaStream_t s, bool tfsf) {
    using G = FusedGeom<T, TY, TZ>;
    const pc_grid_desc& g = c->g;
    FusedState* st = state_of(c);
    bool same = st->ready;
    for (int q = 0; q < 6 && same; ++q) same = st->key_f[0][q] == c->F[0][q] && st->key_f[1][q] == c->F[1][q];
    for (int q = 0; q < 3 && same; ++q) same = st->key_cb[q] == c->cb[q];
    if (!same) {
        for (int set = 0; set < 2; ++set)
            for (int q = 0; q < 3; ++q) {
                int rc = make_map(&st->maps[set].e[q], c->F[set][q], g, G::EW, G::EH);
                if (!rc) rc = make_map(&st->maps[set].h[q], c->F[set][3 + q], g, G::HW, G::HH);
                if (!rc) rc = make_map(&st->maps[set].cb[q], c->cb[q], g, TZ, TY);
                if (rc) return rc;
            }
        for (int q = 0; q < 6; ++q) {
            st->key_f[0][q] = c->F[0][q];
            st->key_f[1][q] = c->F[1][q];
        }
        for (int q = 0; q < 3; ++q) st->key_cb[q] = c->cb[q];
        st->ready = true;
    }
    const int in = c->cur, out = c->cur ^ 1;
    FieldArgs<T> a = make_field_args<T>(c, in, out);
    CpmlArgs<T> p = make_cpml_args<T>(c, in, out);
    const FusedXtra<T> xt = make_fused_xtra<T>(c, tfsf);
    if (p.t > 0 && p.total >= ((int64_t)1 << 31)) return PC_ERR_INVALID;  // 32-bit psi offsets (fused_extras_ok, advance)
    // dynamic shared memory: the stage ring, H^{n+1/2} planes and this grid's CPML table
    const int smem = fused_smem_bytes<T, TY, TZ, S>() + 9 * 2 * std::max(p.t, 1) * (int)sizeof(T);
    const bool cp = p.t > 0, hc = a.da[0] != nullptr, ca = a.ca[0] != nullptr;
    const FusedMaps& m = st->maps[in];
    if (c->fused_cx <= 0) c->fused_cx = choose_chunk<T, TY, TZ, S>(g, smem);
    const int cx = c->fused_cx;
    const int cxe = c->fused_cx_edge > 0 ? c->fused_cx_edge : cx;
    const int kp = (hc ? 2 : 0) | (ca ? 1 : 0);
    // axis-specific classes: float without per-cell H or Ca coefficients (each class
    // is one more kernel instantiation); otherwise every CPML item is general
    const int split = (sizeof(T) == 4 && kp == 0) ? c->fused_split : 0;
    // every class in one launch of fused3_multi (the class in the top byte of w)
    const bool unified = split > 0 && c->fused_unified != 0 && cp;
    if (st->items_cx != cx || st->items_cxe != cxe || st->items_t != p.t || st->items_split != (int)split ||
        st->items_unified != (int)unified || !st->d_items) {
        std::vector<CostItem> cls[CL_N];
        std::vector<int4> all;
        fused_items(g, TY, TZ, cx, cxe, p.t, split, cls);
        if (unified) {
            std::vector<CostItem> merged;
            for (int q = 0; q < CL_N; ++q)
                for (const CostItem& e : cls[q]) merged.push_back({e.first, make_int4(e.second.x, e.second.y,
                                                                                      e.second.z, e.second.w | (q << 24))});
            sort_items(merged);
            for (const CostItem& e : merged) all.push_back(e.second);
            for (int q = 0; q < CL_N; ++q) st->off_cls[q] = st->n_cls[q] = 0;
            st->n_cls[CL_GEN] = (int)all.size();  // launched as one
        } else {
            for (int q = 0; q < CL_N; ++q) {
                st->off_cls[q] = (int)all.size();
                st->n_cls[q] = (int)cls[q].size();
                for (const CostItem& e : cls[q]) all.push_back(e.second);
            }
        }
        cudaFree(st->d_items);
        st->d_items = nullptr;
        PC_CUDA_CHECK(cudaMalloc(&st->d_items, all.size() * sizeof(int4)));
        PC_CUDA_CHECK(cudaMemcpy(st->d_items, all.data(), all.size() * sizeof(int4), cudaMemcpyHostToDevice));
        st->items_cx = cx;
        st->items_cxe = cxe;
        st->items_t = p.t;
        st->items_split = (int)split;
        st->items_unified = (int)unified;
    }
    const int n_plain = st->n_cls[CL_PLAIN];
    int n_side = 0;  // CPML classes with items
    for (int q = CL_GEN; q < CL_N; ++q) n_side += st->n_cls[q] > 0;
    const bool fork = cp && n_side > 0 && (n_plain > 0 || n_side > 1);
    if (fork) {
        if (!st->fork) {
            // highest priority: the slab items are the long ones, so their CTAs are
            // dispatched first and the plain items fill in behind them
            int lo = 0, hi = 0;
            PC_CUDA_CHECK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
            for (int q = 0; q < CL_N - 1; ++q) {
                PC_CUDA_CHECK(cudaStreamCreateWithPriority(&st->side[q], cudaStreamNonBlocking, hi));
                PC_CUDA_CHECK(cudaEventCreateWithFlags(&st->join[q], cudaEventDisableTiming));
            }
            PC_CUDA_CHECK(cudaEventCreateWithFlags(&st->fork, cudaEventDisableTiming));
        }
        PC_CUDA_CHECK(cudaEventRecord(st->fork, s));
    }
    int rc = PC_OK;
    if (cp) {  // the slab classes first (see the side streams' priority)
        for (int q = CL_GEN; q < CL_N && !rc; ++q) {
            const int n = st->n_cls[q];
            if (n <= 0) continue;
            cudaStream_t sq = s;
            if (fork) {
                sq = st->side[q - 1];
                PC_CUDA_CHECK(cudaStreamWaitEvent(sq, st->fork, 0));
            }
            const int4* it = st->d_items + st->off_cls[q];
            if (unified) {
                if constexpr (sizeof(T) == 4) {
                    static bool attr = false;
                    if (!attr) {
                        const int smax = fused_smem_bytes<T, TY, TZ, S>() + 9 * 2 * PC_MAX_CPML * (int)sizeof(T);
                        PC_CUDA_CHECK(cudaFuncSetAttribute(fused3_multi<T, TY, TZ, S, false>,
                                                           cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
                        PC_CUDA_CHECK(cudaFuncSetAttribute(fused3_multi<T, TY, TZ, S, true>,
                                                           cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
                        attr = true;
                    }
                    if (xt.dft.n > 0)
                        fused3_multi<T, TY, TZ, S, true><<<n, dim3(TZ, TY / 2 + 1), smem, sq>>>(a, p, it, m, xt);
                    else
                        fused3_multi<T, TY, TZ, S, false><<<n, dim3(TZ, TY / 2 + 1), smem, sq>>>(a, p, it, m, xt);
                    PC_CUDA_CHECK(cudaGetLastError());
                }
            } else if (q == CL_GEN) {
                switch (kp) {
                    case 0: rc = launch_variant<T, TY, TZ, S, 7, false, false>(sq, a, p, m, xt, smem, it, n); break;
                    case 1: rc = launch_variant<T, TY, TZ, S, 7, false, true>(sq, a, p, m, xt, smem, it, n); break;
                    case 2: rc = launch_variant<T, TY, TZ, S, 7, true, false>(sq, a, p, m, xt, smem, it, n); break;
                    default: rc = launch_variant<T, TY, TZ, S, 7, true, true>(sq, a, p, m, xt, smem, it, n); break;
                }
            } else if constexpr (sizeof(T) == 4) {  // split classes exist only for float, kp == 0
                switch (q) {
                    case CL_YZ: rc = launch_variant<T, TY, TZ, S, 6, false, false>(sq, a, p, m, xt, smem, it, n); break;
                    case CL_XZ: rc = launch_variant<T, TY, TZ, S, 5, false, false>(sq, a, p, m, xt, smem, it, n); break;
                    case CL_XY: rc = launch_variant<T, TY, TZ, S, 3, false, false>(sq, a, p, m, xt, smem, it, n); break;
                    case CL_Z: rc = launch_variant<T, TY, TZ, S, 4, false, false>(sq, a, p, m, xt, smem, it, n); break;
                    case CL_Y: rc = launch_variant<T, TY, TZ, S, 2, false, false>(sq, a, p, m, xt, smem, it, n); break;
                    default: rc = launch_variant<T, TY, TZ, S, 1, false, false>(sq, a, p, m, xt, smem, it, n); break;
                }
            } else {
                rc = PC_ERR_INVALID;
            }
            if (fork) PC_CUDA_CHECK(cudaEventRecord(st->join[q - 1], sq));
            ++c->launches;
        }
        if (rc) return rc;
    }
    // the plain class (no CPML code) on the caller's stream
    const int4* it_plain = st->d_items + st->off_cls[CL_PLAIN];
    switch (kp) {
        case 0: rc = launch_variant<T, TY, TZ, S, 0, false, false>(s, a, p, m, xt, smem, it_plain, n_plain); break;
        case 1: rc = launch_variant<T, TY, TZ, S, 0, false, true>(s, a, p, m, xt, smem, it_plain, n_plain); break;
        case 2: rc = launch_variant<T, TY, TZ, S, 0, true, false>(s, a, p, m, xt, smem, it_plain, n_plain); break;
        default: rc = launch_variant<T, TY, TZ, S, 0, true, true>(s, a, p, m, xt, smem, it_plain, n_plain); break;
    }
    if (rc) return rc;
    if (fork)
        for (int q = CL_GEN; q < CL_N; ++q)
            if (st->n_cls[q] > 0) PC_CUDA_CHECK(cudaStreamWaitEvent(s, st->join[q - 1], 0));
    if (n_plain > 0) ++c->launches;
    c->cur = out;
    return PC_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free stepping (pc_fused_steps_noalloc)
//
// The fused kernel reads its work items from global memory and reports
// non-finite values through a status word.  Callers that may not allocate device
// memory get both from this fixed file-scope array instead: PC_NOALLOC_MAX_ITEMS
// work items followed by one status word (about 512 KB, held by every device that
// loads the library until the process exits).  All calls share it.
// ---------------------------------------------------------------------------
#define PC_NOALLOC_MAX_ITEMS 32768
static __device__ __align__(256) int4 g_noalloc_scratch[PC_NOALLOC_MAX_ITEMS + 1];

// uniform (k-tile, j-tile, chunk) work items, all of equal cost without CPML
__global__ void noalloc_fill_items(int4* items, int ntk, int ntj, int nchunks, int cx, int nx, int TZ_, int TY_,
                                   uint32_t* status) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b == 0) *status = 0u;
    const int n = ntk * ntj * nchunks;
    if (b >= n) return;
    const int kt = b % ntk, jt = (b / ntk) % ntj, ch = b / (ntk * ntj);
    const int ib = ch * cx;
    items[b] = make_int4(kt * TZ_, jt * TY_, ib, min(nx, ib + cx));
}

}  // namespace

namespace {
// Host-side cache of the scratch array's device address, one entry per device
// index, filled on the first call on that device under a lock.  A
// cudaDeviceReset ends the context the address belongs to; the entry is then
// stale and the library must not be called on that device again.
std::mutex g_noalloc_lock;
int g_noalloc_ready[128];
int4* g_noalloc_ptr[128];

template <typename T>
int noalloc_run(int dev, const pc_grid_desc& g, void* const set0[6], void* const set1[6], int cur,
                const void* const cb[3], int nsteps, cudaStream_t s, int4* scratch) {
    constexpr int TY = 16, TZ = 32, S = (sizeof(T) == 4) ? 4 : 3;
    using G = FusedGeom<T, TY, TZ>;
    auto kern = fused3<T, TY, TZ, S, 0, false, false>;
    const int smem = fused_smem_bytes<T, TY, TZ, S>() + 9 * 2 * PC_MAX_CPML * (int)sizeof(T);
    PC_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const int ntk = (g.nz + TZ - 1) / TZ, ntj = (g.ny + TY - 1) / TY;
    // x-chunk: about 8 work items per resident CTA, within the scratch capacity
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TZ * (TY / 2 + 1), smem);
    const double want = 8.0 * (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 1);
    int cx = g.nx;
    const int cands[] = {16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512};
    for (int cand : cands)
        if (cand < g.nx && (double)ntk * ntj * ((g.nx + cand - 1) / cand) >= want) cx = cand;
    int nchunks = (g.nx + cx - 1) / cx;
    while ((int64_t)ntk * ntj * nchunks > PC_NOALLOC_MAX_ITEMS && cx < g.nx) {
        cx *= 2;
        nchunks = (g.nx + cx - 1) / cx;
    }
    const int nitems = ntk * ntj * nchunks;
    if (nitems > PC_NOALLOC_MAX_ITEMS) return PC_ERR_INVALID;  // grid beyond the fixed scratch
    FusedMaps maps[2];
    for (int set = 0; set < 2; ++set) {
        void* const* F = set == 0 ? set0 : set1;
        for (int q = 0; q < 3; ++q) {
            int rc = make_map(&maps[set].e[q], F[q], g, G::EW, G::EH);
            if (!rc) rc = make_map(&maps[set].h[q], F[3 + q], g, G::HW, G::HH);
            if (!rc) rc = make_map(&maps[set].cb[q], cb[q], g, TZ, TY);
            if (rc) return rc;
        }
    }
    int4* items = scratch;
    uint32_t* status = reinterpret_cast<uint32_t*>(scratch + PC_NOALLOC_MAX_ITEMS);
    noalloc_fill_items<<<(nitems + 255) / 256, 256, 0, s>>>(items, ntk, ntj, nchunks, cx, g.nx, TZ, TY, status);
    PC_CUDA_CHECK(cudaGetLastError());
    FieldArgs<T> a{};
    a.nx = g.nx;
    a.ny = g.ny;
    a.nz = g.nz;
    a.pitch = g.pitch;
    a.dx = T(g.dx);
    a.dy = T(g.dy);
    a.dz = T(g.dz);
    a.inv_dx = T(1.0 / g.dx);
    a.inv_dy = T(1.0 / g.dy);
    a.inv_dz = T(1.0 / g.dz);
    a.da_s = T(1.0);
    a.db_s = T((g.dt / (4.0 * M_PI * 1e-7 * 1.0)) / (1.0 + 0.0));  // vacuum mu: dt / mu0
    a.status = status;
    for (int q = 0; q < 3; ++q) a.cb[q] = static_cast<const T*>(cb[q]);
    CpmlArgs<T> pm{};
    for (int n = 0; n < nsteps; ++n) {
        void* const* Fi = cur == 0 ? set0 : set1;
        void* const* Fo = cur == 0 ? set1 : set0;
        for (int q = 0; q < 3; ++q) {
            a.Ein[q] = static_cast<const T*>(Fi[q]);
            a.Hin[q] = static_cast<const T*>(Fi[3 + q]);
            a.Eout[q] = static_cast<T*>(Fo[q]);
            a.Hout[q] = static_cast<T*>(Fo[3 + q]);
        }
        kern<<<nitems, dim3(TZ, TY / 2 + 1), smem, s>>>(a, pm, items, maps[cur], FusedXtra<T>{});
        PC_CUDA_CHECK(cudaGetLastError());
        cur ^= 1;
    }
    return cur;
}
}  // namespace

extern "C" int pc_fused_steps_noalloc(const pc_grid_desc* d, void* const set0[6], void* const set1[6],
                                      int32_t cur, const void* const cb[3], int32_t nsteps, void* stream,
                                      uint32_t* status_out) {
    if (!d || !set0 || !set1 || !cb || nsteps < 0 || (cur != 0 && cur != 1)) return PC_ERR_INVALID;
    if (d->ndim != 3 || d->mode != PC_MODE_CORRECTED || (d->precision != 4 && d->precision != 8))
        return PC_ERR_INVALID;
    if (d->nx < 3 || d->ny < 3 || d->nz < 3 || d->pitch < d->nz || d->pitch % 32 != 0) return PC_ERR_INVALID;
    if ((int64_t)d->nx * d->ny * d->pitch > ((int64_t)1 << 40)) return PC_ERR_INVALID;
    if (!(d->dt > 0) || !(d->dx > 0) || !(d->dy > 0) || !(d->dz > 0)) return PC_ERR_INVALID;
    for (int q = 0; q < 6; ++q)
        if (!set0[q] || !set1[q]) return PC_ERR_INVALID;
    for (int q = 0; q < 3; ++q)
        if (!cb[q]) return PC_ERR_INVALID;
    int dev = 0;
    PC_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return PC_ERR_INVALID;
    int4* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_lock);
        if (!g_noalloc_ready[dev]) {
            // first call on this device (the device is current): resolve the device
            // address of the scratch array; host code may not use the symbol itself
            void* ptr = nullptr;
            PC_CUDA_CHECK(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
            g_noalloc_ptr[dev] = static_cast<int4*>(ptr);
            g_noalloc_ready[dev] = 1;
        }
        scratch = g_noalloc_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int rc = d->precision == 8 ? noalloc_run<double>(dev, *d, set0, set1, cur, cb, nsteps, s, scratch)
                                     : noalloc_run<float>(dev, *d, set0, set1, cur, cb, nsteps, s, scratch);
    if (rc < 0) return rc;
    if (status_out) {
        PC_CUDA_CHECK(cudaMemcpyAsync(status_out, scratch + PC_NOALLOC_MAX_ITEMS, sizeof(uint32_t),
                                      cudaMemcpyDeviceToHost, s));
        PC_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    return rc;
}

bool fused_extras_ok(const pc_ctx* c) {
    const pc_grid_desc& g = c->g;
    if (g.ndim != 3 || g.mode != PC_MODE_CORRECTED || !c->F[1][0]) return false;
    if (g.precision == 4 && (c->ca[0] || c->da[0])) return false;  // those variants leave the extras out
    if (c->cpml_t > 0 && psi_layout(g, c->cpml_t).total >= ((int64_t)1 << 31)) return false;
    if (c->tfsf.on) {
        if (!c->tfsf.d_inc) return false;
        const int k0 = c->tfsf.k0, kH = c->tfsf.dir > 0 ? k0 : k0 + 1;
        if (k0 < 0 || k0 > g.nz - 2 || kH < 1 || kH > g.nz - 2) return false;
        for (int r = 0; r < c->ade_n; ++r)  // the E correction must not precede a pole pass
            if (k0 >= c->ade[r].box[4] && k0 < c->ade[r].box[5]) return false;
    }
    return true;
}

int launch_fused_step(pc_ctx* c, cudaStream_t s, const double* tfsf_amp) {
    if (c->g.ndim != 3) return launch_split_step(c, s);
    if (c->cpml_t > 0 && psi_layout(c->g, c->cpml_t).total >= ((int64_t)1 << 31)) {  // 32-bit psi offsets
        if (c->ade_n > 0 || c->tfsf.on) return PC_ERR_INVALID;
        return launch_split_step(c, s);
    }
    const bool tfsf = c->tfsf.on && tfsf_amp != nullptr;
    if (c->g.precision == 8) return fused_t<double, 16, 32, 3>(c, s, tfsf);
    return fused_t<float, 16, 32, 4>(c, s, tfsf);
}

void destroy_fused_state(pc_ctx* c) {
    if (c->fused_state) {
        FusedState* st = static_cast<FusedState*>(c->fused_state);
        cudaFree(st->d_items);
        for (int q = 0; q < CL_N - 1; ++q) {
            if (st->side[q]) cudaStreamDestroy(st->side[q]);
            if (st->join[q]) cudaEventDestroy(st->join[q]);
        }
        if (st->fork) cudaEventDestroy(st->fork);
    }
    delete static_cast<FusedState*>(c->fused_state);
    c->fused_state = nullptr;
}

}  // namespace pc
