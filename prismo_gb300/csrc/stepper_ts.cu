// Temporally blocked 3D stepper: one launch advances the Yee fields by K = 1 or
// K = 2 whole time steps (float32; Ca = 1, Da = 1 and a scalar Db, i.e. lossless
// non-magnetic media; CPML; soft sources on E fused in).  The update rules are
// those of stepper_split.cu (the reference curls, core/solver.py:167-309, with H
// written one index later), applied in the leap-frog order of
// core/solver.py:535-552 and core/simulation.py:147-164: H^{n+1/2}, E^{n+1}, then
// the sources at t_{n+1}, then the next step.
//
// Work item = a 16 x 32 (j, k) output tile and an x-chunk [ib, ie) of planes.  A
// CTA covers the tile plus K cells on every side (its "region", one point per
// thread) and streams along x.  For every plane p it
//   A  computes H1(p)   from E0(p) (staged by TMA) and its own E0(p-1),
//   B  computes E1(p-1) from H1(p-1) (shared memory) and its own H1(p),
//   C  computes H2(p-1) from E1(p-1) and its own E1(p-2)            (K = 2),
//   D  computes E2(p-2) from H2(p-2) and its own H2(p-1)            (K = 2),
// and stores the last sub-step's H and E of its own tile points.  H needs E at
// j-1 and k-1, E needs H at j+1 and k+1, so every sub-step leaves valid values on
// a region one cell smaller on one side; the region's outer ring holds throw-away
// values that no stored point depends on.  The intermediate state (E1, H1) never
// leaves the SM: with K = 2 one launch reads E, H, Cb and the CPML psi once and
// writes E, H and psi once for two time steps.
//
// E0, H0 and Cb planes of the region arrive through a 4-stage ring of TMA tile
// loads (cp.async.bulk.tensor.3d, one mbarrier per stage, bounded waits); the
// per-plane values a thread needs from earlier planes (own E, H, Cb and psi) stay
// in its registers.  One __syncthreads per plane.  Reads come from field set
// `cur`, writes go to `cur ^ 1`: a neighbouring CTA may still be loading this
// tile's halo.  CPML psi recursions (Roden-Gedney, boundaries/pml.py:117-257
// profiles) run for region points in the slabs; only the owner of a point writes
// its psi.  Items are classified by the slab axes their region reaches and by
// whether it reaches the domain boundary (where the reference's per-component
// update ranges apply); each class runs a body compiled for exactly that case,
// all classes in one launch.
#include <cuda.h>

#include <algorithm>
#include <vector>

#include "pc_internal.cuh"
#include "stencil_common.cuh"
#include "tma.cuh"

namespace pc {

struct TsMaps {
    CUtensorMap e[3];
    CUtensorMap h[3];
    CUtensorMap cb[3];
};

// One fused soft source point on an E component (sources/point.py:62-73 semantics:
// E += w a(t_{n+1}) after the E update of step n).
struct TsSrc {
    int i, j, k, comp;
    double w;
    int col, pad;
};

struct TsArgs {
    int nx, ny, nz, pitch;
    float inv_dx, inv_dy, inv_dz, db;
    float* Eout[3];
    float* Hout[3];
    // CPML (32-bit psi offsets: the host guarantees fewer than 2^31 elements)
    int t;
    int se[3], ab[3];
    int psi_total;
    const float* psi_in;
    float* psi_out;
    const float* slabc;  // [axis][b, a, kinv][2t]
    // fused sources
    const TsSrc* src;
    int nsrc, ns, row0;
    const double* amps;  // [row][ns]
    uint32_t* status;
};

namespace {

constexpr uint32_t kTsWaitLimit = 1u << 22;
constexpr int TS_TY = 16, TS_TZ = 32;
constexpr int TS_BW = TS_TZ + 8;  // TMA box width: k in [k0-4, k0+TZ+4)
constexpr int TS_S = 4;           // stages in the TMA ring

// item classes (the CPML axes a region reaches, and the domain boundary)
enum { TC_PLAIN = 0, TC_EDGE = 1, TC_X = 2, TC_Y = 3, TC_Z = 4, TC_GEN = 5, TC_N = 6 };

template <int K>
struct TsGeom {
    static constexpr int RJ = TS_TY + 2 * K;  // region rows: j in [j0-K, j0+TY+K)
    static constexpr int RK = TS_TZ + 2 * K;  // region columns: k in [k0-K, k0+TZ+K)
    static constexpr int CO = 4 - K;          // box column of region column 0
    static constexpr int NPT = RJ * RK;
    static constexpr int NT = (NPT + 31) / 32 * 32;
    static constexpr int BOXF = RJ * TS_BW;  // floats of one box (one component, one plane)
    static constexpr int BOXB = (BOXF * 4 + 127) / 128 * 128;
    static constexpr int BQ = BOXB / 4;  // box stride in floats
    static constexpr int STAGE = 9 * BOXB;
    static constexpr uint32_t TX = 9u * BOXF * 4u;
    static constexpr int NBUF = K == 2 ? 6 : 2;  // H1 x2 (and E1 x2, H2 x2)
    static constexpr int PAD = 256;              // guard for the outer ring's neighbour reads
    static constexpr int OFF_STAGES = 128 + PAD;
    static constexpr int OFF_BUF = OFF_STAGES + TS_S * STAGE;
    static constexpr int OFF_COEF = OFF_BUF + NBUF * 3 * BOXB;
};

template <int K>
int ts_smem_bytes(int t) {
    using G = TsGeom<K>;
    return G::OFF_COEF + 9 * 2 * std::max(t, 1) * 4 + G::PAD + 128;
}

// one CPML recursion step: psi' = b psi + a d; returns kinv d + psi'
__device__ __forceinline__ float tstep(float b, float a, float kinv, float d, float& psi) {
    psi = b * psi + a * d;
    return d * kinv + psi;
}

// The six psi values of one point for one field (H or E), in derivative order:
// x (slots A, B), y (A, B), z (A, B); see the slot table in pc_internal.cuh.
struct P6 {
    float x0, x1, y0, y1, z0, z1;
};

// Per-thread constants of one region point.
struct TsPt {
    int si;                 // index in a box / buffer plane
    int j, k;               // grid indices
    bool act, own, kjd;     // region point, tile point owned by this CTA, inside the domain
    bool mHx, mHy, mHz, mEx, mEy, mEz;  // j/k part of the update ranges
    int64_t ojk;            // j * pitch + k (owned points)
    int sy, sz;             // y / z slab index (-1: none)
    float yb, ya, yk, zb, za, zk;
    int oxc, oyc, ozc;      // plane-independent parts of the psi offsets
};

__device__ __forceinline__ float psi_ld(const TsArgs& A, int o) {
    if ((unsigned)o < (unsigned)A.psi_total) return __ldg(A.psi_in + o);
    atomicOr(A.status, PC_STATUS_BOUNDS);
    return 0.f;
}
__device__ __forceinline__ void psi_st(const TsArgs& A, int o, float v) {
    if ((unsigned)o < (unsigned)A.psi_total)
        A.psi_out[o] = v;
    else
        atomicOr(A.status, PC_STATUS_BOUNDS);
}

// x-slab index of plane pl (-1: not a slab plane, or no x CPML in this variant)
template <int AX>
__device__ __forceinline__ int x_slab(const TsArgs& A, int t, int pl) {
    if (!(AX & 1) || pl < 0 || pl >= A.nx) return -1;
    return slab_of(pl, A.nx, t);
}

// psi of this point at plane pl (H slots if IS_H, else E slots); sx = x_slab(pl)
template <int AX, bool IS_H>
__device__ __forceinline__ P6 psi_load(const TsArgs& A, const TsPt& pt, int t2, int pl, int sx) {
    P6 v{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (AX == 0 || !pt.act || !pt.kjd || pl < 0 || pl >= A.nx) return v;
    const int P32 = A.pitch, ny = A.ny;
    if ((AX & 1) && sx >= 0) {
        const int o = pt.oxc + sx * (ny * P32);
        v.x0 = psi_ld(A, o + (IS_H ? SX_HY : SX_EY) * A.se[0]);
        v.x1 = psi_ld(A, o + (IS_H ? SX_HZ : SX_EZ) * A.se[0]);
    }
    if ((AX & 2) && pt.sy >= 0) {
        const int o = pt.oyc + pl * (t2 * P32);
        v.y0 = psi_ld(A, o + (IS_H ? SY_HX : SY_EX) * A.se[1]);
        v.y1 = psi_ld(A, o + (IS_H ? SY_HZ : SY_EZ) * A.se[1]);
    }
    if ((AX & 4) && pt.sz >= 0) {
        const int o = pt.ozc + pl * (ny * t2);
        v.z0 = psi_ld(A, o + (IS_H ? SZ_HX : SZ_EX) * A.se[2]);
        v.z1 = psi_ld(A, o + (IS_H ? SZ_HY : SZ_EY) * A.se[2]);
    }
    return v;
}

// the owner's psi at plane pl; u0/u1/u2: whether the x/y/z component of the field
// was updated there (the psi of a component that is not updated is not stored)
template <int AX, bool IS_H>
__device__ __forceinline__ void psi_store(const TsArgs& A, const TsPt& pt, int t2, int pl, int sx, const P6& v,
                                          bool u0, bool u1, bool u2) {
    const int P32 = A.pitch, ny = A.ny;
    // slot -> component: H (Hy Hz | Hx Hz | Hx Hy), E (Ey Ez | Ex Ez | Ex Ey)
    if ((AX & 1) && sx >= 0) {
        const int o = pt.oxc + sx * (ny * P32);
        if (u1) psi_st(A, o + (IS_H ? SX_HY : SX_EY) * A.se[0], v.x0);
        if (u2) psi_st(A, o + (IS_H ? SX_HZ : SX_EZ) * A.se[0], v.x1);
    }
    if ((AX & 2) && pt.sy >= 0) {
        const int o = pt.oyc + pl * (t2 * P32);
        if (u0) psi_st(A, o + (IS_H ? SY_HX : SY_EX) * A.se[1], v.y0);
        if (u2) psi_st(A, o + (IS_H ? SY_HZ : SY_EZ) * A.se[1], v.y1);
    }
    if ((AX & 4) && pt.sz >= 0) {
        const int o = pt.ozc + pl * (ny * t2);
        if (u0) psi_st(A, o + (IS_H ? SZ_HX : SZ_EX) * A.se[2], v.z0);
        if (u1) psi_st(A, o + (IS_H ? SZ_HY : SZ_EY) * A.se[2], v.z1);
    }
}

// H at plane p of this point from E(p) (planes e at stride bq: own value and the
// j-1 / k-1 neighbours) and the point's own E(p-1) (emy, emz).  sx: the plane's x
// slab index, xc: its (b, a, kinv) when sx >= 0.  u: components updated.
template <int AX, bool MASK>
__device__ __forceinline__ void h_upd(const TsArgs& A, const TsPt& pt, const float* e, int bq, float ex, float ey,
                                      float ez, float emy, float emz, int p, int sx, float xb, float xa, float xk,
                                      float& hx, float& hy, float& hz, P6& ps, bool& ux, bool& uy, bool& uz) {
    constexpr int BW = TS_BW;
    const int si = pt.si;
    float d0 = (ez - emz) * A.inv_dx;
    float d1 = (ey - emy) * A.inv_dx;
    float d2 = (ez - e[2 * bq + si - BW]) * A.inv_dy;
    float d3 = (ex - e[si - BW]) * A.inv_dy;
    float d4 = (ey - e[bq + si - 1]) * A.inv_dz;
    float d5 = (ex - e[si - 1]) * A.inv_dz;
    if ((AX & 1) && sx >= 0 && pt.kjd) {
        d0 = tstep(xb, xa, xk, d0, ps.x0);
        d1 = tstep(xb, xa, xk, d1, ps.x1);
    }
    if ((AX & 2) && pt.sy >= 0) {
        d2 = tstep(pt.yb, pt.ya, pt.yk, d2, ps.y0);
        d3 = tstep(pt.yb, pt.ya, pt.yk, d3, ps.y1);
    }
    if ((AX & 4) && pt.sz >= 0) {
        d4 = tstep(pt.zb, pt.za, pt.zk, d4, ps.z0);
        d5 = tstep(pt.zb, pt.za, pt.zk, d5, ps.z1);
    }
    const float db = A.db;
    const float nhx = hx - db * (d2 - d4);
    const float nhy = hy - db * (d5 - d0);
    const float nhz = hz - db * (d1 - d3);
    if (MASK) {
        const bool px = p >= 0 && p <= A.nx - 2, pi = p >= 1 && p <= A.nx - 2;
        ux = pt.mHx && px;
        uy = pt.mHy && pi;
        uz = pt.mHz && pi;
        hx = ux ? nhx : hx;
        hy = uy ? nhy : hy;
        hz = uz ? nhz : hz;
    } else {
        ux = uy = uz = true;
        hx = nhx;
        hy = nhy;
        hz = nhz;
    }
}

// E at plane q of this point from H(q) (planes h at stride bq: the j+1 / k+1
// neighbours), its own H(q) (hxq, hyq, hzq) and H(q+1) (hyn, hzn).
template <int AX, bool MASK>
__device__ __forceinline__ void e_upd(const TsArgs& A, const TsPt& pt, const float* h, int bq, float hxq, float hyq,
                                      float hzq, float hyn, float hzn, int q, int sx, float xb, float xa, float xk,
                                      float cbx, float cby, float cbz, float& ex, float& ey, float& ez, P6& ps,
                                      bool& ux, bool& uy, bool& uz) {
    constexpr int BW = TS_BW;
    const int si = pt.si;
    float d0 = (hzn - hzq) * A.inv_dx;
    float d1 = (hyn - hyq) * A.inv_dx;
    float d2 = (h[2 * bq + si + BW] - hzq) * A.inv_dy;
    float d3 = (h[si + BW] - hxq) * A.inv_dy;
    float d4 = (h[bq + si + 1] - hyq) * A.inv_dz;
    float d5 = (h[si + 1] - hxq) * A.inv_dz;
    if ((AX & 1) && sx >= 0 && pt.kjd) {
        d0 = tstep(xb, xa, xk, d0, ps.x0);
        d1 = tstep(xb, xa, xk, d1, ps.x1);
    }
    if ((AX & 2) && pt.sy >= 0) {
        d2 = tstep(pt.yb, pt.ya, pt.yk, d2, ps.y0);
        d3 = tstep(pt.yb, pt.ya, pt.yk, d3, ps.y1);
    }
    if ((AX & 4) && pt.sz >= 0) {
        d4 = tstep(pt.zb, pt.za, pt.zk, d4, ps.z0);
        d5 = tstep(pt.zb, pt.za, pt.zk, d5, ps.z1);
    }
    const float nex = ex + cbx * (d2 - d4);
    const float ney = ey + cby * (d5 - d0);
    const float nez = ez + cbz * (d1 - d3);
    if (MASK) {
        const bool qd = q >= 0 && q <= A.nx - 1, qi = q >= 0 && q <= A.nx - 2;
        ux = pt.mEx && qd;
        uy = pt.mEy && qi;
        uz = pt.mEz && qi;
        ex = ux ? nex : ex;
        ey = uy ? ney : ey;
        ez = uz ? nez : ez;
    } else {
        ux = uy = uz = true;
        ex = nex;
        ey = ney;
        ez = nez;
    }
}

// fused soft sources of E at plane q, amplitude row `row` of the call
__device__ __forceinline__ void add_src(const TsArgs& A, const TsPt& pt, int q, int row, float& ex, float& ey,
                                        float& ez) {
    for (int m = 0; m < A.nsrc; ++m) {
        const TsSrc S = A.src[m];
        if (S.i == q && S.j == pt.j && S.k == pt.k) {
            const float v = static_cast<float>(S.w * A.amps[(size_t)row * A.ns + S.col]);
            if (S.comp == 0)
                ex = ex + v;
            else if (S.comp == 1)
                ey = ey + v;
            else
                ez = ez + v;
        }
    }
}

// x-slab coefficients (b, a, kinv) of slab index sx (1, 0, 1 off the slabs)
__device__ __forceinline__ void x_coef(const float* sC, int t2, int sx, float& b, float& a, float& kk) {
    b = 1.f, a = 0.f, kk = 1.f;
    if (sx >= 0) {
        b = sC[sx];
        a = sC[t2 + sx];
        kk = sC[2 * t2 + sx];
    }
}

template <int K, int AX, bool MASK>
__device__ __forceinline__ void ts3_item(const TsArgs& A, const TsMaps& maps, const int4 it, unsigned char* smem) {
    using G = TsGeom<K>;
    constexpr bool CP = AX != 0;
    constexpr int BQ = G::BQ;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    unsigned char* stages = smem + G::OFF_STAGES;
    float* buf = reinterpret_cast<float*>(smem + G::OFF_BUF);
    float* sC = reinterpret_cast<float*>(smem + G::OFF_COEF);

    const int tid = threadIdx.x;
    const int k0 = it.x, j0 = it.y, ib = it.z, ie = it.w & 0xFFFFF;
    const bool src_item = ((it.w >> 28) & 1) != 0;
    const int ny = A.ny, nz = A.nz;
    const int pl0 = ib - K;
    const int L = ie - ib + 2 * K;
    const int t = CP ? A.t : 0, t2 = 2 * t;

    if (tid == 0) {
        for (int s = 0; s < TS_S; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
        for (int c = 0; c < 3; ++c) {
            prefetch_tmap(&maps.e[c]);
            prefetch_tmap(&maps.h[c]);
            prefetch_tmap(&maps.cb[c]);
        }
    }
    if (CP)
        for (int i = tid; i < 9 * t2; i += blockDim.x) sC[i] = A.slabc[i];
    __syncthreads();

    auto issue = [&](int n) {
        const int s = n % TS_S;
        unsigned char* st = stages + s * G::STAGE;
        const int pl = pl0 + n;
        mbar_expect_tx(&bars[s], G::TX);
#pragma unroll
        for (int c = 0; c < 3; ++c) tma_load_3d(st + c * G::BOXB, &maps.e[c], k0 - 4, j0 - K, pl, &bars[s]);
#pragma unroll
        for (int c = 0; c < 3; ++c) tma_load_3d(st + (3 + c) * G::BOXB, &maps.h[c], k0 - 4, j0 - K, pl, &bars[s]);
#pragma unroll
        for (int c = 0; c < 3; ++c) tma_load_3d(st + (6 + c) * G::BOXB, &maps.cb[c], k0 - 4, j0 - K, pl, &bars[s]);
    };
    int issued = L < TS_S ? L : TS_S;
    if (tid == 0)
        for (int n = 0; n < issued; ++n) issue(n);

    // ---- this thread's region point -------------------------------------------
    TsPt pt;
    pt.act = tid < G::NPT;
    {
        const int r = pt.act ? tid / G::RK : 0;
        const int c = pt.act ? tid - r * G::RK : 0;
        pt.si = r * TS_BW + c + G::CO;
        pt.j = j0 - K + r;
        pt.k = k0 - K + c;
        pt.own = pt.act && r >= K && r < K + TS_TY && c >= K && c < K + TS_TZ && pt.j < ny && pt.k < nz;
    }
    const int j = pt.j, k = pt.k;
    const int64_t PR = (int64_t)ny * A.pitch;
    pt.ojk = pt.own ? (int64_t)j * A.pitch + k : 0;
    pt.kjd = j >= 0 && j < ny && k >= 0 && k < nz;
    // update ranges of the reference stepper (component shapes, core/grid.py:157-168;
    // H interior, core/solver.py:167-253 with the corrected slices): the j/k parts
    pt.mHx = pt.mHy = pt.mHz = pt.mEx = pt.mEy = pt.mEz = true;
    if (MASK) {
        const bool jd = j >= 0 && j < ny, kd = k >= 0 && k < nz;
        const bool jin = j >= 1 && j <= ny - 2, kin = k >= 1 && k <= nz - 2;
        pt.mHx = jin && kin;
        pt.mHy = jd && j <= ny - 2 && kin;
        pt.mHz = jin && kd && k <= nz - 2;
        pt.mEx = jd && kd && j <= ny - 2 && k <= nz - 2;
        pt.mEy = jd && kd && k <= nz - 2;
        pt.mEz = jd && kd && j <= ny - 2;
    }
    pt.sy = pt.sz = -1;
    pt.yb = pt.yk = pt.zb = pt.zk = 1.f;
    pt.ya = pt.za = 0.f;
    if ((AX & 2) && pt.kjd) {
        pt.sy = slab_of(j, ny, t);
        if (pt.sy >= 0) {
            pt.yb = sC[3 * t2 + pt.sy];
            pt.ya = sC[4 * t2 + pt.sy];
            pt.yk = sC[5 * t2 + pt.sy];
        }
    }
    if ((AX & 4) && pt.kjd) {
        pt.sz = slab_of(k, nz, t);
        if (pt.sz >= 0) {
            pt.zb = sC[6 * t2 + pt.sz];
            pt.za = sC[7 * t2 + pt.sz];
            pt.zk = sC[8 * t2 + pt.sz];
        }
    }
    {
        const int P32 = A.pitch;
        pt.oxc = A.ab[0] + j * P32 + k;
        pt.oyc = A.ab[1] + (pt.sy >= 0 ? pt.sy : 0) * P32 + k;
        pt.ozc = A.ab[2] + j * t2 + (pt.sz >= 0 ? pt.sz : 0);
    }

    float* const H1b0 = buf;
    float* const H1b1 = buf + 3 * BQ;
    float chk = 0.f;  // running sum of the stored E: non-finite iff some value was
    bool timed_out = false;
    int n = 0;
    // carried own values of earlier planes
    float ce0x = 0.f, ce0y = 0.f, ce0z = 0.f;  // E0(p-1)
    float ch1x = 0.f, ch1y = 0.f, ch1z = 0.f;  // H1(p-1)
    float cb1x = 0.f, cb1y = 0.f, cb1z = 0.f;  // Cb(p-1)
    // psi_in of H at plane p and of E at plane p-1, loaded one plane ahead
    P6 pfH = psi_load<AX, true>(A, pt, t2, pl0, x_slab<AX>(A, t, pl0));
    P6 pfE = psi_load<AX, false>(A, pt, t2, pl0 - 1, x_slab<AX>(A, t, pl0 - 1));

    if constexpr (K == 1) {
        for (; n < L; ++n) {
            const int p = pl0 + n, q = p - 1;
            const int s = n % TS_S;
            const bool ok = mbar_wait_bounded(&bars[s], (uint32_t)((n / TS_S) & 1), kTsWaitLimit);
            const float* st = reinterpret_cast<const float*>(stages + s * G::STAGE);
            const int si = pt.si;
            const float e0x = st[si], e0y = st[BQ + si], e0z = st[2 * BQ + si];
            float h1x = st[3 * BQ + si], h1y = st[4 * BQ + si], h1z = st[5 * BQ + si];
            const float cbx = st[6 * BQ + si], cby = st[7 * BQ + si], cbz = st[8 * BQ + si];
            const int sxp = x_slab<AX>(A, t, p), sxq = x_slab<AX>(A, t, q);
            float xbp, xap, xkp, xbq, xaq, xkq;
            x_coef(sC, t2, sxp, xbp, xap, xkp);
            x_coef(sC, t2, sxq, xbq, xaq, xkq);
            P6 psA = pfH, psB = pfE;
            bool ux, uy, uz;
            // A: H1(p)
            h_upd<AX, MASK>(A, pt, st, BQ, e0x, e0y, e0z, ce0y, ce0z, p, sxp, xbp, xap, xkp, h1x, h1y, h1z, psA, ux,
                            uy, uz);
            float* Hw = (n & 1) ? H1b1 : H1b0;
            if (pt.act) {
                Hw[si] = h1x;
                Hw[BQ + si] = h1y;
                Hw[2 * BQ + si] = h1z;
            }
            if (pt.own && p >= ib && p < ie) {
                const int64_t o = (int64_t)p * PR + pt.ojk;
                A.Hout[0][o] = h1x;
                A.Hout[1][o] = h1y;
                A.Hout[2][o] = h1z;
                if (CP) psi_store<AX, true>(A, pt, t2, p, sxp, psA, ux, uy, uz);
            }
            // B: E1(p-1)
            const float* Hr = (n & 1) ? H1b0 : H1b1;
            float e1x = ce0x, e1y = ce0y, e1z = ce0z;
            e_upd<AX, MASK>(A, pt, Hr, BQ, ch1x, ch1y, ch1z, h1y, h1z, q, sxq, xbq, xaq, xkq, cb1x, cb1y, cb1z, e1x,
                            e1y, e1z, psB, ux, uy, uz);
            if (src_item) add_src(A, pt, q, A.row0, e1x, e1y, e1z);
            if (pt.own && q >= ib && q < ie) {
                const int64_t o = (int64_t)q * PR + pt.ojk;
                A.Eout[0][o] = e1x;
                A.Eout[1][o] = e1y;
                A.Eout[2][o] = e1z;
                chk += (e1x + e1y) + e1z;
                if (CP) psi_store<AX, false>(A, pt, t2, q, sxq, psB, ux, uy, uz);
            }
            // next plane's psi, then the carries
            if (CP) {
                pfH = psi_load<AX, true>(A, pt, t2, p + 1, x_slab<AX>(A, t, p + 1));
                pfE = psi_load<AX, false>(A, pt, t2, p, sxp);
            }
            ce0x = e0x, ce0y = e0y, ce0z = e0z;
            ch1x = h1x, ch1y = h1y, ch1z = h1z;
            cb1x = cbx, cb1y = cby, cb1z = cbz;
            if (__syncthreads_or(!ok)) {
                timed_out = true;
                break;
            }
            if (tid == 0 && n + TS_S < L) {
                issue(n + TS_S);
                ++issued;
            }
        }
    } else {
        float* const E1b0 = buf + 6 * BQ;
        float* const E1b1 = buf + 9 * BQ;
        float* const H2b0 = buf + 12 * BQ;
        float* const H2b1 = buf + 15 * BQ;
        float ce1x = 0.f, ce1y = 0.f, ce1z = 0.f;  // E1(p-2)
        float ch2x = 0.f, ch2y = 0.f, ch2z = 0.f;  // H2(p-2)
        float cb2x = 0.f, cb2y = 0.f, cb2z = 0.f;  // Cb(p-2)
        P6 cpH{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};     // psi after step 1: H at p-1
        P6 cpE{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};     // psi after step 1: E at p-2
        for (; n < L; ++n) {
            const int p = pl0 + n, q = p - 1, q2 = p - 2;
            const int s = n % TS_S;
            const bool ok = mbar_wait_bounded(&bars[s], (uint32_t)((n / TS_S) & 1), kTsWaitLimit);
            const float* st = reinterpret_cast<const float*>(stages + s * G::STAGE);
            const int si = pt.si;
            const float e0x = st[si], e0y = st[BQ + si], e0z = st[2 * BQ + si];
            float h1x = st[3 * BQ + si], h1y = st[4 * BQ + si], h1z = st[5 * BQ + si];
            const float cbx = st[6 * BQ + si], cby = st[7 * BQ + si], cbz = st[8 * BQ + si];
            const int sxp = x_slab<AX>(A, t, p), sxq = x_slab<AX>(A, t, q), sxq2 = x_slab<AX>(A, t, q2);
            float xbp, xap, xkp, xbq, xaq, xkq, xbq2, xaq2, xkq2;
            x_coef(sC, t2, sxp, xbp, xap, xkp);
            x_coef(sC, t2, sxq, xbq, xaq, xkq);
            x_coef(sC, t2, sxq2, xbq2, xaq2, xkq2);
            P6 psA = pfH, psB = pfE;
            bool ux, uy, uz;
            // A: H1(p)
            h_upd<AX, MASK>(A, pt, st, BQ, e0x, e0y, e0z, ce0y, ce0z, p, sxp, xbp, xap, xkp, h1x, h1y, h1z, psA, ux,
                            uy, uz);
            float* H1w = (n & 1) ? H1b1 : H1b0;
            if (pt.act) {
                H1w[si] = h1x;
                H1w[BQ + si] = h1y;
                H1w[2 * BQ + si] = h1z;
            }
            // B: E1(p-1)
            const float* H1r = (n & 1) ? H1b0 : H1b1;
            float e1x = ce0x, e1y = ce0y, e1z = ce0z;
            e_upd<AX, MASK>(A, pt, H1r, BQ, ch1x, ch1y, ch1z, h1y, h1z, q, sxq, xbq, xaq, xkq, cb1x, cb1y, cb1z, e1x,
                            e1y, e1z, psB, ux, uy, uz);
            if (src_item) add_src(A, pt, q, A.row0, e1x, e1y, e1z);
            float* E1w = (n & 1) ? E1b0 : E1b1;
            if (pt.act) {
                E1w[si] = e1x;
                E1w[BQ + si] = e1y;
                E1w[2 * BQ + si] = e1z;
            }
            if (__syncthreads_or(!ok)) {
                timed_out = true;
                break;
            }
            if (tid == 0 && n + TS_S < L) {
                issue(n + TS_S);
                ++issued;
            }
            // C: H2(p-1) from E1(p-1) (E1w) and this point's E1(p-2)
            float h2x = ch1x, h2y = ch1y, h2z = ch1z;
            P6 psC = cpH;
            h_upd<AX, MASK>(A, pt, E1w, BQ, e1x, e1y, e1z, ce1y, ce1z, q, sxq, xbq, xaq, xkq, h2x, h2y, h2z, psC, ux,
                            uy, uz);
            float* H2w = (n & 1) ? H2b0 : H2b1;
            if (pt.act) {
                H2w[si] = h2x;
                H2w[BQ + si] = h2y;
                H2w[2 * BQ + si] = h2z;
            }
            if (pt.own && q >= ib && q < ie) {
                const int64_t o = (int64_t)q * PR + pt.ojk;
                A.Hout[0][o] = h2x;
                A.Hout[1][o] = h2y;
                A.Hout[2][o] = h2z;
                if (CP) psi_store<AX, true>(A, pt, t2, q, sxq, psC, ux, uy, uz);
            }
            // D: E2(p-2) from H2(p-2) (written in the previous iteration) and H2(p-1)
            const float* H2r = (n & 1) ? H2b1 : H2b0;
            float e2x = ce1x, e2y = ce1y, e2z = ce1z;
            P6 psD = cpE;
            e_upd<AX, MASK>(A, pt, H2r, BQ, ch2x, ch2y, ch2z, h2y, h2z, q2, sxq2, xbq2, xaq2, xkq2, cb2x, cb2y, cb2z,
                            e2x, e2y, e2z, psD, ux, uy, uz);
            if (src_item) add_src(A, pt, q2, A.row0 + 1, e2x, e2y, e2z);
            if (pt.own && q2 >= ib && q2 < ie) {
                const int64_t o = (int64_t)q2 * PR + pt.ojk;
                A.Eout[0][o] = e2x;
                A.Eout[1][o] = e2y;
                A.Eout[2][o] = e2z;
                chk += (e2x + e2y) + e2z;
                if (CP) psi_store<AX, false>(A, pt, t2, q2, sxq2, psD, ux, uy, uz);
            }
            // next plane's psi, then the carries
            if (CP) {
                pfH = psi_load<AX, true>(A, pt, t2, p + 1, x_slab<AX>(A, t, p + 1));
                pfE = psi_load<AX, false>(A, pt, t2, p, sxp);
                cpH = psA;
                cpE = psB;
            }
            ce0x = e0x, ce0y = e0y, ce0z = e0z;
            ch1x = h1x, ch1y = h1y, ch1z = h1z;
            ce1x = e1x, ce1y = e1y, ce1z = e1z;
            ch2x = h2x, ch2y = h2y, ch2z = h2z;
            cb2x = cb1x, cb2y = cb1y, cb2z = cb1z;
            cb1x = cbx, cb1y = cby, cb1z = cbz;
        }
    }
    if (!isfinite(chk)) atomicOr(A.status, PC_STATUS_NONFINITE);
    if (timed_out) {
        if (tid == 0) atomicOr(A.status, PC_STATUS_TIMEOUT);
        // let every copy already in flight land before the CTA retires
        for (int m = n; m < issued; ++m)
            mbar_wait_bounded(&bars[m % TS_S], (uint32_t)((m / TS_S) & 1), kTsWaitLimit);
    }
}

template <int K>
__global__ void __launch_bounds__(TsGeom<K>::NT, 1)
    ts3_multi(const __grid_constant__ TsArgs A, const __grid_constant__ TsMaps maps, const int4* items) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int4 it = items[blockIdx.x];
    switch ((it.w >> 20) & 7) {
        case TC_PLAIN: ts3_item<K, 0, false>(A, maps, it, smem); break;
        case TC_EDGE: ts3_item<K, 0, true>(A, maps, it, smem); break;
        case TC_X: ts3_item<K, 1, true>(A, maps, it, smem); break;
        case TC_Y: ts3_item<K, 2, true>(A, maps, it, smem); break;
        case TC_Z: ts3_item<K, 4, true>(A, maps, it, smem); break;
        default: ts3_item<K, 7, true>(A, maps, it, smem); break;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct TsState {
    const void* key_f[2][6] = {};
    const void* key_cb[3] = {};
    TsMaps maps[2][2];  // [K - 1][input set]
    bool ready = false;
    int4* d_items[2] = {nullptr, nullptr};
    int nitems[2] = {0, 0}, items_cap[2] = {0, 0};
    int64_t items_key[2][3] = {{-1, -1, -1}, {-1, -1, -1}};  // chunk, t, source generation
    TsSrc* d_src = nullptr;  // TS_MAX_SRC entries
    int nsrc = 0;
    int64_t src_gen = -1;
    bool src_ok = false, src_dirty = false;
    std::vector<TsSrc> hsrc;
};

TsState* ts_of(pc_ctx* c) {
    if (!c->ts_state) c->ts_state = new TsState();
    return static_cast<TsState*>(c->ts_state);
}

// The fused source table: every source point on an E component, with its
// amplitude column; fused only when there are few points (else the separate
// add_sources launch runs after each K = 1 step).
constexpr int TS_MAX_SRC = 64;

int ts_sources(pc_ctx* c, TsState* st) {
    if (st->src_gen == c->gen) return PC_OK;
    st->hsrc.clear();
    bool ok = true;
    size_t total = 0;
    for (const SourceDesc& d : c->sources) total += (size_t)d.n;
    if (total > (size_t)TS_MAX_SRC) ok = false;
    const int64_t P = c->g.pitch, NY = c->g.ny;
    for (size_t q = 0; q < c->sources.size() && ok; ++q) {
        const SourceDesc& d = c->sources[q];
        if (d.comp > 2 || (int)d.h_off.size() != d.n) {
            ok = false;
            break;
        }
        for (int m = 0; m < d.n; ++m) {
            const int64_t o = d.h_off[m];
            TsSrc s{};
            s.i = (int)(o / (NY * P));
            s.j = (int)((o / P) % NY);
            s.k = (int)(o % P);
            s.comp = d.comp;
            s.w = d.h_w[m];
            s.col = (int)q;
            st->hsrc.push_back(s);
        }
    }
    st->src_ok = ok;
    st->nsrc = ok ? (int)st->hsrc.size() : 0;
    st->src_dirty = ok && st->nsrc > 0;
    st->src_gen = c->gen;
    return PC_OK;
}

// Upload a rebuilt source table on the launching stream (ordered after the
// launches that still read the previous one).
int ts_upload_sources(TsState* st, cudaStream_t s) {
    if (!st->src_dirty) return PC_OK;
    if (!st->d_src) {
        PC_CUDA_CHECK(cudaMalloc(&st->d_src, TS_MAX_SRC * sizeof(TsSrc)));
    }
    PC_CUDA_CHECK(cudaMemcpyAsync(st->d_src, st->hsrc.data(), st->nsrc * sizeof(TsSrc), cudaMemcpyHostToDevice, s));
    st->src_dirty = false;
    return PC_OK;
}

// Work items of a chunking for K, classified by what their region and planes reach,
// in spatial order: x-chunk after x-chunk, and within one the tiles row by row, so
// that the CTAs resident at one time hold neighbouring tiles of the same planes and
// the halo rows one of them loads are still in L2 when its neighbours load them.
template <int K>
int ts_items(pc_ctx* c, TsState* st, int cx, cudaStream_t stream) {
    const int ki = K - 1;
    const int t = c->cpml_t;
    if (st->items_key[ki][0] == cx && st->items_key[ki][1] == t && st->items_key[ki][2] == st->src_gen)
        return PC_OK;
    const pc_grid_desc& g = c->g;
    auto touches_slab = [&](int lo, int hi, int n) {  // [lo, hi) against the slabs of an axis of length n
        if (t <= 0) return false;
        const int a = std::max(lo, 0), b = std::min(hi, n);
        return a < b && (a < t || b > n - t);
    };
    auto outside_interior = [&](int lo, int hi, int n) { return lo < 1 || hi > n - 1; };
    std::vector<int4> h;
    for (int ib = 0; ib < g.nx; ib += cx)
        for (int j0 = 0; j0 < g.ny; j0 += TS_TY)
            for (int k0 = 0; k0 < g.nz; k0 += TS_TZ) {
                const int ie = std::min(g.nx, ib + cx);
                const int jlo = j0 - K, jhi = j0 + TS_TY + K, klo = k0 - K, khi = k0 + TS_TZ + K;
                const int plo = ib - K, phi = ie + K;  // planes [plo, phi)
                const bool cxs = touches_slab(plo, phi, g.nx), cys = touches_slab(jlo, jhi, g.ny),
                           czs = touches_slab(klo, khi, g.nz);
                const bool edge = outside_interior(plo, phi, g.nx) || outside_interior(jlo, jhi, g.ny) ||
                                  outside_interior(klo, khi, g.nz);
                const int axes = (cxs ? 1 : 0) + (cys ? 1 : 0) + (czs ? 1 : 0);
                int cls;
                if (axes == 0)
                    cls = edge ? TC_EDGE : TC_PLAIN;
                else if (axes == 1)
                    cls = cxs ? TC_X : (cys ? TC_Y : TC_Z);
                else
                    cls = TC_GEN;
                bool src = false;
                for (const TsSrc& s : st->hsrc)
                    src = src || (s.i >= plo && s.i < phi && s.j >= jlo && s.j < jhi && s.k >= klo && s.k < khi);
                const int w = ie | (cls << 20) | ((src && st->src_ok) ? (1 << 28) : 0);
                h.push_back(make_int4(k0, j0, ib, w));
            }
    if ((int)h.size() > st->items_cap[ki]) {
        cudaFree(st->d_items[ki]);  // synchronises the device: no launch still reads it
        st->d_items[ki] = nullptr;
        st->items_cap[ki] = 0;
        PC_CUDA_CHECK(cudaMalloc(&st->d_items[ki], h.size() * sizeof(int4)));
        st->items_cap[ki] = (int)h.size();
    }
    // pageable source: the copy is staged before this call returns, and runs in
    // stream order after the launches that read the previous table
    PC_CUDA_CHECK(cudaMemcpyAsync(st->d_items[ki], h.data(), h.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                  stream));
    st->nitems[ki] = (int)h.size();
    st->items_key[ki][0] = cx;
    st->items_key[ki][1] = t;
    st->items_key[ki][2] = st->src_gen;
    return PC_OK;
}

template <int K>
int ts_launch(pc_ctx* c, int row, cudaStream_t s, bool* fused_sources) {
    using G = TsGeom<K>;
    const pc_grid_desc& g = c->g;
    TsState* st = ts_of(c);
    bool same = st->ready;
    for (int q = 0; q < 6 && same; ++q) same = st->key_f[0][q] == c->F[0][q] && st->key_f[1][q] == c->F[1][q];
    for (int q = 0; q < 3 && same; ++q) same = st->key_cb[q] == c->cb[q];
    if (!same) {
        for (int kk = 0; kk < 2; ++kk)
            for (int set = 0; set < 2; ++set)
                for (int q = 0; q < 3; ++q) {
                    const int rows = TS_TY + 2 * (kk + 1);
                    int rc = make_map(&st->maps[kk][set].e[q], c->F[set][q], g, TS_BW, rows);
                    if (!rc) rc = make_map(&st->maps[kk][set].h[q], c->F[set][3 + q], g, TS_BW, rows);
                    if (!rc) rc = make_map(&st->maps[kk][set].cb[q], c->cb[q], g, TS_BW, rows);
                    if (rc) return rc;
                }
        for (int q = 0; q < 6; ++q) {
            st->key_f[0][q] = c->F[0][q];
            st->key_f[1][q] = c->F[1][q];
        }
        for (int q = 0; q < 3; ++q) st->key_cb[q] = c->cb[q];
        st->ready = true;
    }
    int rc = ts_sources(c, st);
    if (!rc) rc = ts_upload_sources(st, s);
    if (rc) return rc;
    const int cx = c->ts_cx > 0 ? std::min(c->ts_cx, g.nx) : std::min(32, g.nx);
    rc = ts_items<K>(c, st, cx, s);
    if (rc) return rc;
    const int in = c->cur, out = c->cur ^ 1;
    TsArgs A{};
    A.nx = g.nx;
    A.ny = g.ny;
    A.nz = g.nz;
    A.pitch = g.pitch;
    A.inv_dx = (float)(1.0 / g.dx);
    A.inv_dy = (float)(1.0 / g.dy);
    A.inv_dz = (float)(1.0 / g.dz);
    A.db = (float)c->db_s;
    for (int q = 0; q < 3; ++q) {
        A.Eout[q] = static_cast<float*>(c->F[out][q]);
        A.Hout[q] = static_cast<float*>(c->F[out][3 + q]);
    }
    A.t = c->cpml_t;
    if (A.t > 0) {
        const PsiLayout Lp = psi_layout(g, A.t);
        if (Lp.total >= ((int64_t)1 << 31)) return PC_ERR_INVALID;
        for (int q = 0; q < 3; ++q) {
            A.se[q] = (int)Lp.slot_elems[q];
            A.ab[q] = (int)Lp.axis_base[q];
        }
        A.psi_total = (int)Lp.total;
        A.psi_in = static_cast<const float*>(c->psi[in] ? c->psi[in] : c->psi[0]);
        A.psi_out = static_cast<float*>(c->psi[out] ? c->psi[out] : c->psi[0]);
        A.slabc = static_cast<const float*>(c->d_cpml_slab);
    }
    const bool fs = st->src_ok && st->nsrc > 0;
    A.src = fs ? st->d_src : nullptr;
    A.nsrc = fs ? st->nsrc : 0;
    A.ns = (int)c->sources.size();
    A.row0 = row;
    A.amps = c->d_amps;
    A.status = c->d_status;
    *fused_sources = fs || c->sources.empty();
    const int smem = ts_smem_bytes<K>(A.t);
    auto kern = ts3_multi<K>;
    static bool attr = false;
    if (!attr) {
        PC_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, ts_smem_bytes<K>(PC_MAX_CPML)));
        attr = true;
    }
    kern<<<st->nitems[K - 1], G::NT, smem, s>>>(A, st->maps[K - 1][in], st->d_items[K - 1]);
    PC_CUDA_CHECK(cudaGetLastError());
    ++c->launches;
    c->cur = out;
    return PC_OK;
}

}  // namespace

bool ts_eligible(const pc_ctx* c) {
    const pc_grid_desc& g = c->g;
    if (c->ts_k <= 0 || g.ndim != 3 || g.precision != 4 || g.mode != PC_MODE_CORRECTED) return false;
    if (g.sched != PC_SCHED_FUSED || c->ade_n > 0 || c->tfsf.on) return false;
    for (int q = 0; q < 3; ++q)
        if (c->ca[q] || c->da[q] || c->db[q] || !c->cb[q]) return false;
    if (g.nx < 3 || g.ny < 3 || g.nz < 3 || !c->F[1][0]) return false;
    if (c->cpml_t > 0 && (psi_layout(g, c->cpml_t).total >= ((int64_t)1 << 31) || !c->d_cpml_slab)) return false;
    return (int64_t)g.nx * g.ny * g.pitch < ((int64_t)1 << 40);
}

// K = 2 also needs every per-step consumer of the fields to be absent (monitors
// sample after each step) and its sources fused.
bool ts_two_step_ok(pc_ctx* c) {
    if (c->ts_k < 2 || !ts_eligible(c)) return false;
    if (!c->dfts.empty() || !c->fluxes.empty() || !c->modes.empty()) return false;
    if (c->sources.empty()) return true;
    TsState* st = ts_of(c);
    if (ts_sources(c, st) != PC_OK) return false;
    return st->src_ok;
}

int launch_ts_step(pc_ctx* c, int k, int row, cudaStream_t s, bool* fused_sources) {
    return k == 2 ? ts_launch<2>(c, row, s, fused_sources) : ts_launch<1>(c, row, s, fused_sources);
}

void destroy_ts_state(pc_ctx* c) {
    if (!c->ts_state) return;
    TsState* st = static_cast<TsState*>(c->ts_state);
    for (int q = 0; q < 2; ++q) cudaFree(st->d_items[q]);
    cudaFree(st->d_src);
    delete st;
    c->ts_state = nullptr;
}

}  // namespace pc
