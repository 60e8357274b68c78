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
    static constexpr int RK = TS_TZ + 4;      // region columns: k in [k0-2, k0+TZ+2) (pairs stay aligned)
    static constexpr int CO = 2;              // box column of region column 0
    static constexpr int NPR = RK / 2;        // k-pairs per region row
    static constexpr int NPAIR = RJ * NPR;    // one pair of points per thread
    static constexpr int NT = (NPAIR + 31) / 32 * 32;
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

// Per-point constants (one of the two points a thread owns).
struct TsPc {
    int k;
    bool kjd;                           // inside the domain
    bool mHx, mHy, mHz, mEx, mEy, mEz;  // j/k part of the update ranges
    int sz;                             // z slab index (-1: none)
    float zb, za, zk;
    int oxc, oyc, ozc;                  // plane-independent parts of the psi offsets
};

// Coefficients shared by the points of a row: y slab (index and b, a, kinv).
struct TsRow {
    int sy;
    float yb, ya, yk;
};

// x-slab index of plane pl (-1: not a slab plane, or no x CPML in this variant)
template <int AX>
__device__ __forceinline__ int x_slab(const TsArgs& A, int t, int pl) {
    if (!(AX & 1) || pl < 0 || pl >= A.nx) return -1;
    return slab_of(pl, A.nx, t);
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

// Plane part of the update ranges and the x-slab state of one plane (uniform).
struct TsPlane {
    bool hx, hi;  // H: plane in [0, nx-2] / [1, nx-2]
    bool ed, ei;  // E: plane in [0, nx-1] / [0, nx-2]
    int sx;       // x slab index (-1: none)
    float xb, xa, xk;
};

template <int AX>
__device__ __forceinline__ TsPlane plane_of(const TsArgs& A, const float* sC, int t, int pl) {
    TsPlane P;
    P.hx = pl >= 0 && pl <= A.nx - 2;
    P.hi = pl >= 1 && pl <= A.nx - 2;
    P.ed = pl >= 0 && pl <= A.nx - 1;
    P.ei = P.hx;
    P.sx = x_slab<AX>(A, t, pl);
    x_coef(sC, 2 * t, P.sx, P.xb, P.xa, P.xk);
    return P;
}

// psi of one point at plane pl (H slots if IS_H, else E slots); sx = x_slab(pl).
// Offsets were range-checked once per work item (psi_ok).
template <int AX, bool IS_H>
__device__ __forceinline__ P6 psi_load(const TsArgs& A, const TsPc& pc, int sy, bool ok, int t2, int pl, int sx) {
    P6 v{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (AX == 0 || !ok || !pc.kjd || pl < 0 || pl >= A.nx) return v;
    const int P32 = A.pitch, ny = A.ny;
    const float* in = A.psi_in;
    if ((AX & 1) && sx >= 0) {
        const int o = pc.oxc + sx * (ny * P32);
        v.x0 = __ldg(in + o + (IS_H ? SX_HY : SX_EY) * A.se[0]);
        v.x1 = __ldg(in + o + (IS_H ? SX_HZ : SX_EZ) * A.se[0]);
    }
    if ((AX & 2) && sy >= 0) {
        const int o = pc.oyc + pl * (t2 * P32);
        v.y0 = __ldg(in + o + (IS_H ? SY_HX : SY_EX) * A.se[1]);
        v.y1 = __ldg(in + o + (IS_H ? SY_HZ : SY_EZ) * A.se[1]);
    }
    if ((AX & 4) && pc.sz >= 0) {
        const int o = pc.ozc + pl * (ny * t2);
        v.z0 = __ldg(in + o + (IS_H ? SZ_HX : SZ_EX) * A.se[2]);
        v.z1 = __ldg(in + o + (IS_H ? SZ_HY : SZ_EY) * A.se[2]);
    }
    return v;
}

// the owner's psi at plane pl; u0/u1/u2: whether the x/y/z component of the field
// was updated there (the psi of a component that is not updated is not stored)
template <int AX, bool IS_H>
__device__ __forceinline__ void psi_store(const TsArgs& A, const TsPc& pc, int sy, int t2, int pl, int sx,
                                          const P6& v, bool u0, bool u1, bool u2) {
    if (!pc.kjd) return;
    const int P32 = A.pitch, ny = A.ny;
    float* out = A.psi_out;
    // slot -> component: H (Hy Hz | Hx Hz | Hx Hy), E (Ey Ez | Ex Ez | Ex Ey)
    if ((AX & 1) && sx >= 0) {
        const int o = pc.oxc + sx * (ny * P32);
        if (u1) out[o + (IS_H ? SX_HY : SX_EY) * A.se[0]] = v.x0;
        if (u2) out[o + (IS_H ? SX_HZ : SX_EZ) * A.se[0]] = v.x1;
    }
    if ((AX & 2) && sy >= 0) {
        const int o = pc.oyc + pl * (t2 * P32);
        if (u0) out[o + (IS_H ? SY_HX : SY_EX) * A.se[1]] = v.y0;
        if (u2) out[o + (IS_H ? SY_HZ : SY_EZ) * A.se[1]] = v.y1;
    }
    if ((AX & 4) && pc.sz >= 0) {
        const int o = pc.ozc + pl * (ny * t2);
        if (u0) out[o + (IS_H ? SZ_HX : SZ_EX) * A.se[2]] = v.z0;
        if (u1) out[o + (IS_H ? SZ_HY : SZ_EY) * A.se[2]] = v.z1;
    }
}

// H at plane p of one point: own E(p) (ex, ey, ez), neighbours Ez, Ex at j-1 and
// Ey, Ex at k-1, own E(p-1) (emy, emz).  px / pi: the plane lies in [0, nx-2] /
// [1, nx-2]; use_psi: the point or the plane lies in a slab; sx / (xb, xa, xk):
// the plane's x slab.
template <int AX, bool MASK>
__device__ __forceinline__ void h_point(const TsArgs& A, const TsPc& pc, const TsRow& rw, float ex, float ey, float ez,
                                        float ezj, float exj, float eyk, float exk, float emy, float emz, bool px,
                                        bool pi, bool use_psi, int sx, float xb, float xa, float xk, float& hx,
                                        float& hy, float& hz, P6& ps, bool& ux, bool& uy, bool& uz) {
    float d0 = (ez - emz) * A.inv_dx;
    float d1 = (ey - emy) * A.inv_dx;
    float d2 = (ez - ezj) * A.inv_dy;
    float d3 = (ex - exj) * A.inv_dy;
    float d4 = (ey - eyk) * A.inv_dz;
    float d5 = (ex - exk) * A.inv_dz;
    if (AX != 0 && use_psi) {
        if ((AX & 1) && sx >= 0 && pc.kjd) {
            d0 = tstep(xb, xa, xk, d0, ps.x0);
            d1 = tstep(xb, xa, xk, d1, ps.x1);
        }
        if ((AX & 2) && rw.sy >= 0 && pc.kjd) {
            d2 = tstep(rw.yb, rw.ya, rw.yk, d2, ps.y0);
            d3 = tstep(rw.yb, rw.ya, rw.yk, d3, ps.y1);
        }
        if ((AX & 4) && pc.sz >= 0) {
            d4 = tstep(pc.zb, pc.za, pc.zk, d4, ps.z0);
            d5 = tstep(pc.zb, pc.za, pc.zk, d5, ps.z1);
        }
    }
    const float db = A.db;
    const float nhx = hx - db * (d2 - d4);
    const float nhy = hy - db * (d5 - d0);
    const float nhz = hz - db * (d1 - d3);
    if (MASK) {
        ux = pc.mHx && px;
        uy = pc.mHy && pi;
        uz = pc.mHz && pi;
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

// E at plane q of one point: neighbours Hz, Hx at j+1 and Hy, Hx at k+1, own H(q)
// (hxq, hyq, hzq) and H(q+1) (hyn, hzn), Cb (cbx, cby, cbz).  qd / qi: the plane
// lies in [0, nx-1] / [0, nx-2].
template <int AX, bool MASK>
__device__ __forceinline__ void e_point(const TsArgs& A, const TsPc& pc, const TsRow& rw, float hzj, float hxj,
                                        float hyk, float hxk, float hxq, float hyq, float hzq, float hyn, float hzn,
                                        bool qd, bool qi, bool use_psi, int sx, float xb, float xa, float xk,
                                        float cbx, float cby, float cbz, float& ex, float& ey, float& ez, P6& ps,
                                        bool& ux, bool& uy, bool& uz) {
    float d0 = (hzn - hzq) * A.inv_dx;
    float d1 = (hyn - hyq) * A.inv_dx;
    float d2 = (hzj - hzq) * A.inv_dy;
    float d3 = (hxj - hxq) * A.inv_dy;
    float d4 = (hyk - hyq) * A.inv_dz;
    float d5 = (hxk - hxq) * A.inv_dz;
    if (AX != 0 && use_psi) {
        if ((AX & 1) && sx >= 0 && pc.kjd) {
            d0 = tstep(xb, xa, xk, d0, ps.x0);
            d1 = tstep(xb, xa, xk, d1, ps.x1);
        }
        if ((AX & 2) && rw.sy >= 0 && pc.kjd) {
            d2 = tstep(rw.yb, rw.ya, rw.yk, d2, ps.y0);
            d3 = tstep(rw.yb, rw.ya, rw.yk, d3, ps.y1);
        }
        if ((AX & 4) && pc.sz >= 0) {
            d4 = tstep(pc.zb, pc.za, pc.zk, d4, ps.z0);
            d5 = tstep(pc.zb, pc.za, pc.zk, d5, ps.z1);
        }
    }
    const float nex = ex + cbx * (d2 - d4);
    const float ney = ey + cby * (d5 - d0);
    const float nez = ez + cbz * (d1 - d3);
    if (MASK) {
        ux = pc.mEx && qd;
        uy = pc.mEy && qi;
        uz = pc.mEz && qi;
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

// fused soft sources of E at plane q, point (j, k), amplitude row `row` of the call
__device__ __forceinline__ void add_src(const TsArgs& A, int j, int k, int q, int row, float& ex, float& ey,
                                        float& ez) {
    for (int m = 0; m < A.nsrc; ++m) {
        const TsSrc S = A.src[m];
        if (S.i == q && S.j == j && S.k == k) {
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

__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }

// Field values of a pair of points (.x: the point at k, .y: the one at k+1).
struct V3 {
    float2 x, y, z;
};
__device__ __forceinline__ V3 ld3(const float* b, int bq, int si) {
    return V3{ld2(b + si), ld2(b + bq + si), ld2(b + 2 * bq + si)};
}
__device__ __forceinline__ void st3(float* b, int bq, int si, const V3& v) {
    st2(b + si, v.x.x, v.x.y);
    st2(b + bq + si, v.y.x, v.y.y);
    st2(b + 2 * bq + si, v.z.x, v.z.y);
}

// H sub-step of a pair at plane P: E(p) planes e (own pair and neighbours), own
// E(p-1) (em), H in/out (h).
template <int AX, bool MASK>
__device__ __forceinline__ void h_pair(const TsArgs& A, const TsPc* pc, const TsRow& rw, const float* e, int bq, int si,
                                       const V3& eo, const V3& em, const TsPlane& P, bool use_psi, V3& h, P6* ps,
                                       bool* u) {
    constexpr int BW = TS_BW;
    const float2 ezj = ld2(e + 2 * bq + si - BW), exj = ld2(e + si - BW);
    const float eyk = e[bq + si - 1], exk = e[si - 1];
    h_point<AX, MASK>(A, pc[0], rw, eo.x.x, eo.y.x, eo.z.x, ezj.x, exj.x, eyk, exk, em.y.x, em.z.x, P.hx, P.hi,
                      use_psi, P.sx, P.xb, P.xa, P.xk, h.x.x, h.y.x, h.z.x, ps[0], u[0], u[1], u[2]);
    h_point<AX, MASK>(A, pc[1], rw, eo.x.y, eo.y.y, eo.z.y, ezj.y, exj.y, eo.y.x, eo.x.x, em.y.y, em.z.y, P.hx, P.hi,
                      use_psi, P.sx, P.xb, P.xa, P.xk, h.x.y, h.y.y, h.z.y, ps[1], u[3], u[4], u[5]);
}

// E sub-step of a pair at plane P: H(q) planes h (neighbours), own H(q) (hq) and
// H(q+1) (hn), Cb (cb), E in/out (e).
template <int AX, bool MASK>
__device__ __forceinline__ void e_pair(const TsArgs& A, const TsPc* pc, const TsRow& rw, const float* h, int bq, int si,
                                       const V3& hq, const V3& hn, const V3& cb, const TsPlane& P, bool use_psi, V3& e,
                                       P6* ps, bool* u) {
    constexpr int BW = TS_BW;
    const float2 hzj = ld2(h + 2 * bq + si + BW), hxj = ld2(h + si + BW);
    const float hyk = h[bq + si + 2], hxk = h[si + 2];
    e_point<AX, MASK>(A, pc[0], rw, hzj.x, hxj.x, hq.y.y, hq.x.y, hq.x.x, hq.y.x, hq.z.x, hn.y.x, hn.z.x, P.ed, P.ei,
                      use_psi, P.sx, P.xb, P.xa, P.xk, cb.x.x, cb.y.x, cb.z.x, e.x.x, e.y.x, e.z.x, ps[0], u[0], u[1],
                      u[2]);
    e_point<AX, MASK>(A, pc[1], rw, hzj.y, hxj.y, hyk, hxk, hq.x.y, hq.y.y, hq.z.y, hn.y.y, hn.z.y, P.ed, P.ei,
                      use_psi, P.sx, P.xb, P.xa, P.xk, cb.x.y, cb.y.y, cb.z.y, e.x.y, e.y.y, e.z.y, ps[1], u[3], u[4],
                      u[5]);
}

// Region row r and pair column u of thread `tid` (< RJ * NPR).  Each half-warp
// takes the 16 inner pair columns (u = 1..16, 32 consecutive floats) of one row,
// so its float2 shared-memory accesses touch 32 distinct banks; the two outer
// columns of every row (u = 0, NPR - 1) follow, two per thread pair.  (A plain
// row-major order puts 18 pairs in a row: half-warps straddling two rows then
// hit the same banks twice.  Packing the z-slab pairs of a CPML item first, so
// that fewer warps run the z recursions, measured slower than this order: 85.0
// against 88.0 Gcell/s at 256^3.)
template <int K>
__device__ __forceinline__ void pair_of(int tid, int& r, int& u) {
    constexpr int NPR = TsGeom<K>::NPR, RJ = TsGeom<K>::RJ, NM = NPR - 2;
    static_assert(NM == 16, "a half-warp spans the inner pair columns of a row");
    if (tid < RJ * NM) {
        r = tid / NM;
        u = 1 + (tid - r * NM);
    } else {
        const int v = tid - RJ * NM;
        r = v >> 1;
        u = (v & 1) ? NPR - 1 : 0;
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

    // ---- this thread's pair of region points ----------------------------------
    const bool act = tid < G::NPAIR;
    int r = 0, u = 0;
    if (act) pair_of<K>(tid, r, u);
    const int si = r * TS_BW + 2 * u + G::CO;  // even: float2 accesses stay aligned
    const int j = j0 - K + r;
    const int kp = k0 - 2 + 2 * u;  // the pair's first k (even when k0 is)
    const bool own = act && r >= K && r < K + TS_TY && u >= 1 && u <= TS_TZ / 2 && j < ny && kp < nz;
    const int64_t PR = (int64_t)ny * A.pitch;
    const int64_t ojk = own ? (int64_t)j * A.pitch + kp : 0;
    TsRow rw;
    rw.sy = -1;
    rw.yb = rw.yk = 1.f;
    rw.ya = 0.f;
    const bool jd = j >= 0 && j < ny;
    if ((AX & 2) && jd) {
        rw.sy = slab_of(j, ny, t);
        if (rw.sy >= 0) {
            rw.yb = sC[3 * t2 + rw.sy];
            rw.ya = sC[4 * t2 + rw.sy];
            rw.yk = sC[5 * t2 + rw.sy];
        }
    }
    TsPc pc[2];
    bool psi_ok = true;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        TsPc& c = pc[h];
        const int k = kp + h;
        c.k = k;
        c.kjd = act && jd && k >= 0 && k < nz;
        // update ranges of the reference stepper (component shapes, core/grid.py:157-168;
        // H interior, core/solver.py:167-253 with the corrected slices): the j/k parts
        c.mHx = c.mHy = c.mHz = c.mEx = c.mEy = c.mEz = true;
        if (MASK) {
            const bool kd = k >= 0 && k < nz;
            const bool jin = j >= 1 && j <= ny - 2, kin = k >= 1 && k <= nz - 2;
            c.mHx = jin && kin;
            c.mHy = jd && j <= ny - 2 && kin;
            c.mHz = jin && kd && k <= nz - 2;
            c.mEx = jd && kd && j <= ny - 2 && k <= nz - 2;
            c.mEy = jd && kd && k <= nz - 2;
            c.mEz = jd && kd && j <= ny - 2;
        }
        c.sz = -1;
        c.zb = c.zk = 1.f;
        c.za = 0.f;
        if ((AX & 4) && c.kjd) {
            c.sz = slab_of(k, nz, t);
            if (c.sz >= 0) {
                c.zb = sC[6 * t2 + c.sz];
                c.za = sC[7 * t2 + c.sz];
                c.zk = sC[8 * t2 + c.sz];
            }
        }
        const int P32 = A.pitch;
        c.oxc = A.ab[0] + j * P32 + k;
        c.oyc = A.ab[1] + (rw.sy >= 0 ? rw.sy : 0) * P32 + k;
        c.ozc = A.ab[2] + j * t2 + (c.sz >= 0 ? c.sz : 0);
        if (CP && c.kjd) {
            // every psi offset this point forms over the item's planes, checked once:
            // x-slab entries at any slab index, y/z-slab entries up to the last plane
            const int64_t last = min(ie + K, A.nx) - 1;
            const int64_t tot = A.psi_total;
            bool ok = true;
            if (AX & 1) ok = ok && c.oxc >= 0 && (int64_t)c.oxc + (int64_t)(t2 - 1) * ny * P32 + 3LL * A.se[0] < tot;
            if ((AX & 2) && rw.sy >= 0) ok = ok && c.oyc >= 0 && (int64_t)c.oyc + last * t2 * P32 + 3LL * A.se[1] < tot;
            if ((AX & 4) && c.sz >= 0) ok = ok && c.ozc >= 0 && (int64_t)c.ozc + last * ny * t2 + 3LL * A.se[2] < tot;
            psi_ok = psi_ok && ok;
        }
    }
    if (CP && !psi_ok) atomicOr(A.status, PC_STATUS_BOUNDS);  // psi traffic of this pair is skipped
    // psi work only where this pair or the plane lies in a slab (warp-uniform for
    // the x slabs)
    const bool yzs = CP && psi_ok &&
                     (((AX & 2) && rw.sy >= 0 && (pc[0].kjd || pc[1].kjd)) || ((AX & 4) && (pc[0].sz >= 0 || pc[1].sz >= 0)));
    auto use_psi = [&](const TsPlane& P) { return CP && psi_ok && (yzs || P.sx >= 0); };

    float* const H1b0 = buf;
    float* const H1b1 = buf + 3 * BQ;
    float chk = 0.f;  // running sum of the stored E: non-finite iff some value was
    bool timed_out = false;
    int n = 0;
    const float2 z2 = make_float2(0.f, 0.f);
    // carried own values of earlier planes
    V3 ce0{z2, z2, z2};  // E0(p-1)
    V3 ch1{z2, z2, z2};  // H1(p-1)
    V3 cb1{z2, z2, z2};  // Cb(p-1)
    // psi_in of H at plane p and of E at plane p-1, loaded one plane ahead
    P6 pfH[2], pfE[2];
    TsPlane Pn = plane_of<AX>(A, sC, t, pl0);  // plane p of the next iteration
    TsPlane Pq = plane_of<AX>(A, sC, t, pl0 - 1);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        pfH[h] = pfE[h] = P6{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (use_psi(Pn)) pfH[h] = psi_load<AX, true>(A, pc[h], rw.sy, psi_ok, t2, pl0, Pn.sx);
        if (use_psi(Pq)) pfE[h] = psi_load<AX, false>(A, pc[h], rw.sy, psi_ok, t2, pl0 - 1, Pq.sx);
    }
    bool uu[6];

    if constexpr (K == 1) {
        for (; n < L; ++n) {
            const int p = pl0 + n, q = p - 1;
            const int s = n % TS_S;
            const bool ok = mbar_wait_bounded(&bars[s], (uint32_t)((n / TS_S) & 1), kTsWaitLimit);
            const float* st = reinterpret_cast<const float*>(stages + s * G::STAGE);
            const V3 e0 = ld3(st, BQ, si);
            V3 h1 = ld3(st + 3 * BQ, BQ, si);
            const V3 cb = ld3(st + 6 * BQ, BQ, si);
            const TsPlane Pp = Pn;  // plane p
            const bool psp = use_psi(Pp), psq = use_psi(Pq);
            // A: H1(p)
            h_pair<AX, MASK>(A, pc, rw, st, BQ, si, e0, ce0, Pp, psp, h1, pfH, uu);
            float* Hw = (n & 1) ? H1b1 : H1b0;
            if (act) st3(Hw, BQ, si, h1);
            if (own && p >= ib && p < ie) {
                const int64_t o = (int64_t)p * PR + ojk;
                st2(A.Hout[0] + o, h1.x.x, h1.x.y);
                st2(A.Hout[1] + o, h1.y.x, h1.y.y);
                st2(A.Hout[2] + o, h1.z.x, h1.z.y);
                if (psp) {
                    psi_store<AX, true>(A, pc[0], rw.sy, t2, p, Pp.sx, pfH[0], uu[0], uu[1], uu[2]);
                    psi_store<AX, true>(A, pc[1], rw.sy, t2, p, Pp.sx, pfH[1], uu[3], uu[4], uu[5]);
                }
            }
            // B: E1(p-1)
            const float* Hr = (n & 1) ? H1b0 : H1b1;
            V3 e1 = ce0;
            e_pair<AX, MASK>(A, pc, rw, Hr, BQ, si, ch1, h1, cb1, Pq, psq, e1, pfE, uu);
            if (src_item) {
                add_src(A, j, kp, q, A.row0, e1.x.x, e1.y.x, e1.z.x);
                add_src(A, j, kp + 1, q, A.row0, e1.x.y, e1.y.y, e1.z.y);
            }
            if (own && q >= ib && q < ie) {
                const int64_t o = (int64_t)q * PR + ojk;
                st2(A.Eout[0] + o, e1.x.x, e1.x.y);
                st2(A.Eout[1] + o, e1.y.x, e1.y.y);
                st2(A.Eout[2] + o, e1.z.x, e1.z.y);
                chk += ((e1.x.x + e1.y.x) + e1.z.x) + ((e1.x.y + e1.y.y) + e1.z.y);
                if (psq) {
                    psi_store<AX, false>(A, pc[0], rw.sy, t2, q, Pq.sx, pfE[0], uu[0], uu[1], uu[2]);
                    psi_store<AX, false>(A, pc[1], rw.sy, t2, q, Pq.sx, pfE[1], uu[3], uu[4], uu[5]);
                }
            }
            // next plane's state and psi, then the carries
            Pn = plane_of<AX>(A, sC, t, p + 1);
            Pq = Pp;
            if (CP) {
                const bool psn = use_psi(Pn);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (psn) pfH[h] = psi_load<AX, true>(A, pc[h], rw.sy, psi_ok, t2, p + 1, Pn.sx);
                    if (psp) pfE[h] = psi_load<AX, false>(A, pc[h], rw.sy, psi_ok, t2, p, Pp.sx);
                }
            }
            ce0 = e0;
            ch1 = h1;
            cb1 = cb;
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
        V3 ce1{z2, z2, z2};  // E1(p-2)
        V3 ch2{z2, z2, z2};  // H2(p-2)
        V3 cb2{z2, z2, z2};  // Cb(p-2)
        P6 cpH[2], cpE[2];   // psi after step 1: H at p-1, E at p-2
#pragma unroll
        for (int h = 0; h < 2; ++h) cpH[h] = cpE[h] = P6{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        TsPlane Pq2 = plane_of<AX>(A, sC, t, pl0 - 2);
        for (; n < L; ++n) {
            const int p = pl0 + n, q = p - 1, q2 = p - 2;
            const int s = n % TS_S;
            const bool ok = mbar_wait_bounded(&bars[s], (uint32_t)((n / TS_S) & 1), kTsWaitLimit);
            const float* st = reinterpret_cast<const float*>(stages + s * G::STAGE);
            const V3 e0 = ld3(st, BQ, si);
            V3 h1 = ld3(st + 3 * BQ, BQ, si);
            const V3 cb = ld3(st + 6 * BQ, BQ, si);
            const TsPlane Pp = Pn;  // plane p (Pq: p-1, Pq2: p-2)
            const bool psp = use_psi(Pp), psq = use_psi(Pq), psq2 = use_psi(Pq2);
            // A: H1(p)
            h_pair<AX, MASK>(A, pc, rw, st, BQ, si, e0, ce0, Pp, psp, h1, pfH, uu);
            float* H1w = (n & 1) ? H1b1 : H1b0;
            if (act) st3(H1w, BQ, si, h1);
            // B: E1(p-1)
            const float* H1r = (n & 1) ? H1b0 : H1b1;
            V3 e1 = ce0;
            e_pair<AX, MASK>(A, pc, rw, H1r, BQ, si, ch1, h1, cb1, Pq, psq, e1, pfE, uu);
            if (src_item) {
                add_src(A, j, kp, q, A.row0, e1.x.x, e1.y.x, e1.z.x);
                add_src(A, j, kp + 1, q, A.row0, e1.x.y, e1.y.y, e1.z.y);
            }
            float* E1w = (n & 1) ? E1b0 : E1b1;
            if (act) st3(E1w, BQ, si, e1);
            if (__syncthreads_or(!ok)) {
                timed_out = true;
                break;
            }
            if (tid == 0 && n + TS_S < L) {
                issue(n + TS_S);
                ++issued;
            }
            // C: H2(p-1) from E1(p-1) (E1w) and this pair's E1(p-2)
            V3 h2 = ch1;
            h_pair<AX, MASK>(A, pc, rw, E1w, BQ, si, e1, ce1, Pq, psq, h2, cpH, uu);
            float* H2w = (n & 1) ? H2b0 : H2b1;
            if (act) st3(H2w, BQ, si, h2);
            if (own && q >= ib && q < ie) {
                const int64_t o = (int64_t)q * PR + ojk;
                st2(A.Hout[0] + o, h2.x.x, h2.x.y);
                st2(A.Hout[1] + o, h2.y.x, h2.y.y);
                st2(A.Hout[2] + o, h2.z.x, h2.z.y);
                if (psq) {
                    psi_store<AX, true>(A, pc[0], rw.sy, t2, q, Pq.sx, cpH[0], uu[0], uu[1], uu[2]);
                    psi_store<AX, true>(A, pc[1], rw.sy, t2, q, Pq.sx, cpH[1], uu[3], uu[4], uu[5]);
                }
            }
            // D: E2(p-2) from H2(p-2) (written in the previous iteration) and H2(p-1)
            const float* H2r = (n & 1) ? H2b1 : H2b0;
            V3 e2 = ce1;
            e_pair<AX, MASK>(A, pc, rw, H2r, BQ, si, ch2, h2, cb2, Pq2, psq2, e2, cpE, uu);
            if (src_item) {
                add_src(A, j, kp, q2, A.row0 + 1, e2.x.x, e2.y.x, e2.z.x);
                add_src(A, j, kp + 1, q2, A.row0 + 1, e2.x.y, e2.y.y, e2.z.y);
            }
            if (own && q2 >= ib && q2 < ie) {
                const int64_t o = (int64_t)q2 * PR + ojk;
                st2(A.Eout[0] + o, e2.x.x, e2.x.y);
                st2(A.Eout[1] + o, e2.y.x, e2.y.y);
                st2(A.Eout[2] + o, e2.z.x, e2.z.y);
                chk += ((e2.x.x + e2.y.x) + e2.z.x) + ((e2.x.y + e2.y.y) + e2.z.y);
                if (psq2) {
                    psi_store<AX, false>(A, pc[0], rw.sy, t2, q2, Pq2.sx, cpE[0], uu[0], uu[1], uu[2]);
                    psi_store<AX, false>(A, pc[1], rw.sy, t2, q2, Pq2.sx, cpE[1], uu[3], uu[4], uu[5]);
                }
            }
            // next plane's state and psi, then the carries
            Pq2 = Pq;
            Pq = Pp;
            Pn = plane_of<AX>(A, sC, t, p + 1);
            if (CP) {
                const bool psn = use_psi(Pn);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (psp) cpH[h] = pfH[h];  // H psi of plane p after step 1
                    if (psq) cpE[h] = pfE[h];  // E psi of plane p-1 after step 1
                    if (psn) pfH[h] = psi_load<AX, true>(A, pc[h], rw.sy, psi_ok, t2, p + 1, Pn.sx);
                    if (psp) pfE[h] = psi_load<AX, false>(A, pc[h], rw.sy, psi_ok, t2, p, Pp.sx);
                }
            }
            ce0 = e0;
            ch1 = h1;
            ce1 = e1;
            ch2 = h2;
            cb2 = cb1;
            cb1 = cb;
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
    int64_t items_key[2][4] = {{-1, -1, -1, -1}, {-1, -1, -1, -1}};  // chunk, t, source generation, order
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
    if (st->items_key[ki][0] == cx && st->items_key[ki][1] == t && st->items_key[ki][2] == st->src_gen &&
        st->items_key[ki][3] == c->ts_order)
        return PC_OK;
    const pc_grid_desc& g = c->g;
    auto touches_slab = [&](int lo, int hi, int n) {  // [lo, hi) against the slabs of an axis of length n
        if (t <= 0) return false;
        const int a = std::max(lo, 0), b = std::min(hi, n);
        return a < b && (a < t || b > n - t);
    };
    auto outside_interior = [&](int lo, int hi, int n) { return lo < 1 || hi > n - 1; };
    static const float kCost[TC_N] = {1.0f, 1.2f, 1.8f, 1.8f, 1.8f, 2.5f};  // relative time per plane
    std::vector<int4> h;
    std::vector<float> cost;
    std::vector<int> chunk;
    // x-chunk boundaries: with an x CPML the end chunks cover the slab and the K
    // planes beyond it, so that the chunks between them (whose K halo planes then
    // stay clear of the slab) run without x-CPML code; cx elsewhere
    std::vector<int> bounds{0};
    {
        const int edge_len = t + K;
        const bool split_ends = t > 0 && g.nx > 2 * edge_len + 2 * K;
        int ib = 0;
        if (split_ends) {
            ib = edge_len;
            bounds.push_back(ib);
        }
        const int stop = split_ends ? g.nx - edge_len : g.nx;
        while (ib < stop) {
            ib = std::min(stop, ib + cx);
            bounds.push_back(ib);
        }
        if (split_ends) bounds.push_back(g.nx);
    }
    for (size_t ci = 0; ci + 1 < bounds.size(); ++ci)
        for (int j0 = 0; j0 < g.ny; j0 += TS_TY)
            for (int k0 = 0; k0 < g.nz; k0 += TS_TZ) {
                const int ib = bounds[ci], ie = bounds[ci + 1];
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
                cost.push_back(kCost[cls] * (float)(ie - ib + 2 * K));
                chunk.push_back((int)ci);
            }
    if (c->ts_order != 0) {
        // order 1: x-chunks by their summed cost, most expensive first (the slab
        // chunks), and within a chunk the slower items first; the tiles of one
        // chunk still run together (one chunk is about one wave of CTAs), so their
        // shared halo rows are read from L2.  order 2: every item by cost.
        const int nch = (int)bounds.size() - 1;
        std::vector<float> csum(nch, 0.f);
        for (size_t q = 0; q < h.size(); ++q) csum[chunk[q]] += cost[q];
        std::vector<int> ord(h.size());
        for (size_t q = 0; q < ord.size(); ++q) ord[q] = (int)q;
        const bool by_item = c->ts_order == 2;
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
            if (!by_item && chunk[a] != chunk[b]) {
                if (csum[chunk[a]] != csum[chunk[b]]) return csum[chunk[a]] > csum[chunk[b]];
                return chunk[a] < chunk[b];
            }
            return cost[a] > cost[b];
        });
        std::vector<int4> o(h.size());
        for (size_t q = 0; q < ord.size(); ++q) o[q] = h[ord[q]];
        h.swap(o);
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
    st->items_key[ki][3] = c->ts_order;
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
