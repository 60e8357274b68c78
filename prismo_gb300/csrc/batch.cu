// Batched 2D sweep engine: many uneven 2D TE simulations (Ez, Hx, Hy: the
// reference's "TE mode", core/solver.py:311-456 with the corrected stencil)
// advanced together by persistent kernels.
//
// The reference runs a parameter sweep one design after another
// (optimization/sweep.py:41-195, each design a full Simulation.run).  Here every
// design of a sweep is an *instance* whose Ez/Hx/Hy live in shared device buffers
// at per-instance offsets; a host-built work table lists (instance, tile) items
// and persistent grids of CTAs walk it.
//
// One pass advances every instance by K steps (temporal blocking): a CTA loads
// its tile plus a K-cell halo of Ez, Hx, Hy into shared memory, runs K leap-frog
// steps there (the valid region shrinks by one cell per side per step), and
// writes the tile interior to the other field set (ping-pong).  Every thread owns
// y-adjacent cell pairs and keeps them in registers across the K steps; shared
// memory carries the values neighbouring threads read.  Items fall in three
// classes, each with its own kernel: tiles whose region lies inside the instance
// and clear of the CPML, the source column and the port lines take a branch-free
// path (no per-cell tests, three shared arrays); tiles at the instance edges or on
// the CPML keep per-cell flags (components the stepper does not update there, slab
// indices) and the four CPML auxiliaries in shared memory, with their y-slab pairs
// ordered first so that only the warps holding them run the psi code; tiles with
// source or port cells add, on top of that, the soft mode-profile line source in
// the E phase (sources/point.py:62-73 semantics, amplitude at t_{n+1}) and sample
// the port DFT lines into the shared DFT ring.  The time loop is captured once as
// a CUDA graph of G steps and replayed; a device step counter drives the amplitude
// table.
//
// Arithmetic per point is that of the single-simulation 2D stepper (stepper_split.cu
// split_h2 / split_e2 Ez family), with every rounding explicit so that every
// class and every tile shape give the same bits.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "pc_internal.cuh"

namespace pc {
namespace {

constexpr int BNT = 512;  // threads per CTA
constexpr int RING_T = 16;
constexpr int PC_MAX_BATCH_CPML = 100;  // slab thickness limit (shared-memory coefficient table)

struct BInst {  // device copy of one instance (128 bytes)
    int nx, ny, pitch, src_x;
    int src_y0, src_n, nport, pad0;
    int64_t f_off, c_off, p_off, w_off;
    int mx[4], my0[4], mn[4], mpt[4];
};
static_assert(sizeof(BInst) == 128, "BInst layout");

struct BPass {
    const BInst* inst;
    const int4* items;  // (instance, x0, y0, flags)
    int nitems;
    const float* fin;
    float* fout;
    const float* cb;
    const float* psi_in;
    float* psi_out;
    const float* slab;  // [3][2t]: b, a, 1/kappa by slab index
    int t;
    float inv_dx, inv_dy, da, db;
    const double* amps;
    int namps;
    const long long* step;  // device step counter (steps completed before this chunk)
    int s_off;              // first step of this pass relative to *step
    int row0;               // DFT ring row of the first step of this pass
    float* ring;
    int npts;
    const double* w;  // source weights
    int live;         // 0: dry pass (no source, no sampling) used by the tuner
    unsigned* status;       // batch status word
    unsigned* inst_status;  // [ninst] per-instance status words
};

// Non-finite sentinel of one item: `chk` is the sum of the Ez values this thread
// stored; NaN or Inf marks the item's instance (and the batch) failed.
__device__ __forceinline__ void flag_nonfinite(const BPass& P, int inst, float chk) {
    if (!isfinite(chk)) {
        atomicOr(P.inst_status + inst, PC_STATUS_NONFINITE);
        atomicOr(P.status, PC_STATUS_NONFINITE);
    }
}

enum : unsigned {
    F_HX = 1u,
    F_HY = 2u,
    F_EZ = 4u,
    F_INT = 8u,
    F_SRC = 16u,
    F_PORT = 32u,
    F_IN = 64u,
};

__device__ __forceinline__ int slab_idx(int idx, int n, int t) {
    return idx < t ? idx : (idx >= n - t ? idx - (n - 2 * t) : 255);
}

// per-thread cells of a (TX + 2K) x (TY + 2K) region
template <int TX, int TY, int K>
struct BShape {
    static_assert(TY % 2 == 0, "the fast path moves y-adjacent pairs");
    static constexpr int RX = TX + 2 * K, RY = TY + 2 * K, RC = RX * RY, M = (RC + BNT - 1) / BNT;
    static constexpr int MP = (RC / 2 + BNT - 1) / BNT;  // cell pairs per thread
    // two CTAs per SM (64 registers a thread) while a thread's pairs, flags and psi
    // offsets fit; the fast path three (42 registers) for at most two pairs
    static constexpr int MINB = M <= 8 ? 2 : 1;
    static constexpr int MINB_FAST = MP <= 2 ? 3 : (MP <= 8 ? 2 : 1);
    // Ez, Hx, Hy with RY + 2 guard cells on both sides (edge cells read their
    // neighbours without tests), then (edge and source/port items) the four CPML
    // auxiliaries
    static constexpr int GUARD = RY + 2;  // even: the float2 accesses stay 8-byte aligned
    static constexpr int FS = RC + 2 * GUARD;
    static constexpr size_t SMEM = sizeof(float) * (3 * FS + 4 * RC);
    static constexpr size_t SMEM_FAST = sizeof(float) * 3 * FS;
};

// The update formulas with explicit rounding (no contraction choices left to the
// compiler), so that every item class -- and therefore every tile shape -- gives
// bit-identical fields.  Same operations as split_h2 / split_e2.
__device__ __forceinline__ float cpml_d(float d, float b, float a, float kinv, float& psi) {
    psi = __fmaf_rn(b, psi, __fmul_rn(a, d));
    return __fmaf_rn(d, kinv, psi);
}
__device__ __forceinline__ float h_minus(float h, float d, float da, float db) {  // Hx: da h - db d
    return __fmaf_rn(-db, d, __fmul_rn(da, h));
}
__device__ __forceinline__ float h_plus(float h, float d, float da, float db) {  // Hy: da h + db d
    return __fmaf_rn(db, d, __fmul_rn(da, h));
}
__device__ __forceinline__ float diff(float a, float b, float inv) { return __fmul_rn(__fsub_rn(a, b), inv); }

// FAST: the kernel of the fast-path items (their own table and launch, with the
// smaller shared-memory footprint and higher occupancy); otherwise the edge / CPML
// items, SPEC: those holding source or port cells (the only ones that compile the
// source and port-sample code; their own table and launch as well).
template <int TX, int TY, int K, bool FAST, bool SPEC>
__global__ void __launch_bounds__(BNT, FAST ? BShape<TX, TY, K>::MINB_FAST : BShape<TX, TY, K>::MINB)
    batch2d_pass(BPass P) {
    using SH = BShape<TX, TY, K>;
    constexpr int RX = SH::RX, RY = SH::RY, RC = SH::RC;
    constexpr int M = SH::M;
    extern __shared__ float smem[];
    float* sE = smem + SH::GUARD;
    float* sX = sE + SH::FS;
    float* sY = sX + SH::FS;
    float* qYX = smem + 3 * SH::FS;  // psi of Hy (x-derivative)
    float* qZX = qYX + RC;           // psi of Ez (x-derivative)
    float* qXY = qZX + RC;           // psi of Hx (y-derivative)
    float* qZY = qXY + RC;           // psi of Ez (y-derivative)
    __shared__ BInst sI;
    __shared__ float sC[3 * 2 * PC_MAX_BATCH_CPML];  // b, a, 1/kappa by slab index
    const int tid = threadIdx.x;
    const long long base = P.live ? *P.step : 0;
    const int t = P.t;
    for (int q = tid; q < 6 * t; q += BNT) sC[q] = P.slab[q];
    const float* sb = sC;
    const float* sa = sC + 2 * t;
    const float* sk = sC + 4 * t;
    const float idx_ = P.inv_dx, idy = P.inv_dy, da = P.da, db = P.db;

    for (int w = blockIdx.x; w < P.nitems; w += gridDim.x) {
        const int4 it = P.items[w];
        __syncthreads();  // the previous item is done with shared memory
        if (tid < 32) reinterpret_cast<int*>(&sI)[tid] = reinterpret_cast<const int*>(P.inst + it.x)[tid];
        __syncthreads();
        const int nx = sI.nx, ny = sI.ny;
        const int64_t pitch = sI.pitch;
        const int64_t nxp = (int64_t)nx * pitch;
        const int gx0 = it.y - K, gy0 = it.z - K;
        const bool cp = it.w & 1;
        const float* fin = P.fin + sI.f_off;
        float* fout = P.fout + sI.f_off;
        const float* cbp = P.cb + sI.c_off;
        if (FAST) {
            // ---- fast path: the region lies inside the instance, clear of the CPML,
            // the source column and the port lines: every cell updates every component
            // (edge cells read guard or wrapped neighbours; their results fall outside
            // the shrinking valid region and are never stored).  Each thread owns pairs
            // of y-adjacent cells and moves them as float2.
            constexpr int NP = RC / 2;
            constexpr int MP = (NP + BNT - 1) / BNT;
            // this thread's pairs stay in registers across the K steps; shared memory
            // carries only what neighbouring threads read
            float2 cb2[MP], er[MP], xr[MP], yr[MP];
#pragma unroll
            for (int m = 0; m < MP; ++m) {
                const int q = tid + m * BNT;
                cb2[m] = er[m] = xr[m] = yr[m] = make_float2(0.f, 0.f);
                if (q >= NP) continue;
                const int idx = 2 * q;
                const int r = idx / RY, c = idx - (idx / RY) * RY;
                const int64_t o = (int64_t)(gx0 + r) * pitch + (gy0 + c);
                if (K % 2 == 0) {  // o is even: 8-byte aligned pairs
                    er[m] = *reinterpret_cast<const float2*>(fin + o);
                    xr[m] = *reinterpret_cast<const float2*>(fin + nxp + o);
                    yr[m] = *reinterpret_cast<const float2*>(fin + 2 * nxp + o);
                    cb2[m] = *reinterpret_cast<const float2*>(cbp + o);
                } else {
                    er[m] = make_float2(fin[o], fin[o + 1]);
                    xr[m] = make_float2(fin[nxp + o], fin[nxp + o + 1]);
                    yr[m] = make_float2(fin[2 * nxp + o], fin[2 * nxp + o + 1]);
                    cb2[m] = make_float2(cbp[o], cbp[o + 1]);
                }
                *reinterpret_cast<float2*>(sE + idx) = er[m];
                *reinterpret_cast<float2*>(sX + idx) = xr[m];
                *reinterpret_cast<float2*>(sY + idx) = yr[m];
            }
            __syncthreads();
#pragma unroll
            for (int s = 0; s < K; ++s) {
#pragma unroll
                for (int m = 0; m < MP; ++m) {
                    const int q = tid + m * BNT;
                    if (q >= NP) continue;
                    const int idx = 2 * q;
                    const float2 e = er[m];
                    const float2 eu = *reinterpret_cast<const float2*>(sE + idx - RY);
                    const float em = sE[idx - 1];
                    float2 hx = xr[m], hy = yr[m];
                    hx.x = h_minus(hx.x, diff(e.x, em, idy), da, db);
                    hx.y = h_minus(hx.y, diff(e.y, e.x, idy), da, db);
                    hy.x = h_plus(hy.x, diff(e.x, eu.x, idx_), da, db);
                    hy.y = h_plus(hy.y, diff(e.y, eu.y, idx_), da, db);
                    xr[m] = hx;
                    yr[m] = hy;
                    *reinterpret_cast<float2*>(sX + idx) = hx;
                    *reinterpret_cast<float2*>(sY + idx) = hy;
                }
                __syncthreads();
#pragma unroll
                for (int m = 0; m < MP; ++m) {
                    const int q = tid + m * BNT;
                    if (q >= NP) continue;
                    const int idx = 2 * q;
                    const float2 hx = xr[m], hy = yr[m];
                    const float2 hyd = *reinterpret_cast<const float2*>(sY + idx + RY);
                    const float hxn = sX[idx + 2];
                    float2 e = er[m];
                    e.x = __fmaf_rn(cb2[m].x, __fsub_rn(diff(hyd.x, hy.x, idx_), diff(hx.y, hx.x, idy)), e.x);
                    e.y = __fmaf_rn(cb2[m].y, __fsub_rn(diff(hyd.y, hy.y, idx_), diff(hxn, hx.y, idy)), e.y);
                    er[m] = e;
                    *reinterpret_cast<float2*>(sE + idx) = e;
                }
                __syncthreads();
            }
            float chk = 0.f;
#pragma unroll
            for (int m = 0; m < MP; ++m) {
                const int q = tid + m * BNT;
                if (q >= NP) continue;
                const int idx = 2 * q;
                const int r = idx / RY, c = idx - (idx / RY) * RY;
                if (r < K || r >= K + TX) continue;
                const int64_t o = (int64_t)(gx0 + r) * pitch + (gy0 + c);
                if (K % 2 == 0) {  // c even, K and TY even: both cells of the pair are in or out
                    if (c < K || c >= K + TY) continue;
                    *reinterpret_cast<float2*>(fout + o) = er[m];
                    *reinterpret_cast<float2*>(fout + nxp + o) = xr[m];
                    *reinterpret_cast<float2*>(fout + 2 * nxp + o) = yr[m];
                    chk += er[m].x + er[m].y;
                } else {
                    const float ev[2] = {er[m].x, er[m].y}, xv[2] = {xr[m].x, xr[m].y}, yv[2] = {yr[m].x, yr[m].y};
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        if (c + h < K || c + h >= K + TY) continue;
                        fout[o + h] = ev[h];
                        fout[nxp + o + h] = xv[h];
                        fout[2 * nxp + o + h] = yv[h];
                        chk += ev[h];
                    }
                }
            }
            flag_nonfinite(P, it.x, chk);
            continue;
        }
        const int64_t pyx = sI.p_off;                      // psi Hy (x-derivative), [2t][pitch]
        const int64_t pzx = pyx + 2 * (int64_t)t * pitch;  // psi Ez (x-derivative), [2t][pitch]
        const int64_t pxy = pyx + 4 * (int64_t)t * pitch;  // psi Hx (y-derivative), [nx][2t]
        const int64_t pzy = pxy + 2 * (int64_t)t * nx;     // psi Ez (y-derivative), [nx][2t]
        {
            // ---- paired path of the other items: at the instance edges or on the CPML
            // slabs, and (SPEC) holding source or port cells.  The fast path's y-adjacent pairs and guard cells
            // (region-edge cells compute garbage that never reaches the shrinking valid
            // region), plus per-cell flags only where the stencil of the reference
            // stepper differs: components it does not update at the instance edges keep
            // their value (a select, so even the sign of a zero is kept), the psi
            // recursions run on slab cells that update, cells outside the instance load
            // as zero and are never stored.
            constexpr int NP = RC / 2;
            constexpr int MP = (NP + BNT - 1) / BNT;
            float2 cb2[MP], er[MP], xr[MP], yr[MP];  // own pairs stay in registers
            unsigned fl2[2 * MP];
            // Pair order: the pairs of the y-slab columns first (row by row), then the
            // others, so that the psi code of a y-edge tile runs in the warps that hold
            // slab pairs only, not in every warp of the tile.  [a0, b0) and [a1, b1):
            // the region's slab pair columns (low and high y slab, possibly empty).
            constexpr int NPC = RY / 2;  // pairs per row
            int pidx[MP];
            {
                const int a0 = max(0, -gy0) / 2, b0 = max(a0, min(RY, t - gy0) / 2 + (min(RY, t - gy0) & 1));
                const int lo1 = max(max(0, ny - t - gy0), 2 * b0), hi1 = min(RY, ny - gy0);
                const int a1 = lo1 / 2, b1 = max(a1, hi1 / 2 + (hi1 & 1));
                const int ns = (b0 - a0) + (b1 - a1), nn = NPC - ns;
#pragma unroll
                for (int m = 0; m < MP; ++m) {
                    const int q = tid + m * BNT;
                    int r = 0, c2 = 0;
                    if (q < RX * ns) {
                        r = q / ns;
                        const int k = q - r * ns;
                        c2 = k < b0 - a0 ? a0 + k : a1 + (k - (b0 - a0));
                    } else if (q < NP) {
                        const int qq = q - RX * ns;
                        r = qq / nn;
                        const int k = qq - r * nn;  // k-th column outside [a0, b0) and [a1, b1)
                        c2 = k < a0 ? k : (k - a0 + b0 < a1 ? k - a0 + b0 : k - a0 - (a1 - b0) + b1);
                    }
                    pidx[m] = r * RY + 2 * c2;
                }
            }
            // fl2, per cell: bit 0 Hx, 1 Hy, 2 Ez updates, 3 interior, 4 source cell,
            // 5 port cell; x slab index << 8, y slab index << 16 (255: none)
#pragma unroll
            for (int m = 0; m < MP; ++m) {
                const int q = tid + m * BNT;
                cb2[m] = er[m] = xr[m] = yr[m] = make_float2(0.f, 0.f);
                fl2[2 * m] = fl2[2 * m + 1] = (255u << 8) | (255u << 16);
                if (q >= NP) continue;
                const int idx = pidx[m];
                const int r = idx / RY, c0 = idx - (idx / RY) * RY;
                const int gi = gx0 + r;
                float cbv[2], ev[2], xv[2], yv[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int c = c0 + h, gj = gy0 + c;
                    const bool in = gi >= 0 && gi < nx && gj >= 0 && gj < ny;
                    float e = 0.f, hx = 0.f, hy = 0.f;
                    cbv[h] = 0.f;
                    unsigned f = 0, sxs = 255, sys = 255;
                    if (in) {
                        const int64_t o = (int64_t)gi * pitch + gj;
                        e = fin[o];
                        hx = fin[nxp + o];
                        hy = fin[2 * nxp + o];
                        cbv[h] = cbp[o];
                        if (gi < nx - 1 && gj >= 1 && gj <= ny - 2) f |= 1u;
                        if (gi >= 1 && gi <= nx - 2 && gj < ny - 1) f |= 2u;
                        if (gi < nx - 1 && gj < ny - 1) f |= 4u;
                        if (r >= K && r < K + TX && c >= K && c < K + TY) f |= 8u;
                        if (SPEC && gi == sI.src_x && (unsigned)(gj - sI.src_y0) < (unsigned)sI.src_n) f |= 16u;
                        if (SPEC && (f & 8u))
                            for (int q2 = 0; q2 < sI.nport; ++q2)
                                if (gi == sI.mx[q2] && (unsigned)(gj - sI.my0[q2]) < (unsigned)sI.mn[q2]) f |= 32u;
                        if (cp) {
                            sxs = slab_idx(gi, nx, t);
                            sys = slab_idx(gj, ny, t);
                            if (sxs != 255) {
                                qYX[idx + h] = P.psi_in[pyx + (int64_t)sxs * pitch + gj];
                                qZX[idx + h] = P.psi_in[pzx + (int64_t)sxs * pitch + gj];
                            }
                            if (sys != 255) {
                                qXY[idx + h] = P.psi_in[pxy + (int64_t)gi * (2 * t) + sys];
                                qZY[idx + h] = P.psi_in[pzy + (int64_t)gi * (2 * t) + sys];
                            }
                        }
                    }
                    fl2[2 * m + h] = f | (sxs << 8) | (sys << 16);
                    sE[idx + h] = e;
                    sX[idx + h] = hx;
                    sY[idx + h] = hy;
                    ev[h] = e;
                    xv[h] = hx;
                    yv[h] = hy;
                }
                cb2[m] = make_float2(cbv[0], cbv[1]);
                er[m] = make_float2(ev[0], ev[1]);
                xr[m] = make_float2(xv[0], xv[1]);
                yr[m] = make_float2(yv[0], yv[1]);
            }
            __syncthreads();
#pragma unroll 1
            for (int s = 0; s < K; ++s) {
                double amp = 0.0;  // the source amplitude a(t_{n+1}) of this step
                if (SPEC && P.live) {
                    const long long n = base + P.s_off + s;
                    if (n < P.namps) amp = P.amps[n];
                }
#pragma unroll
                for (int m = 0; m < MP; ++m) {
                    const int q = tid + m * BNT;
                    if (q >= NP) continue;
                    const int idx = pidx[m];
                    const float2 e = er[m];
                    const float2 eu = *reinterpret_cast<const float2*>(sE + idx - RY);
                    const float em = sE[idx - 1];
                    float2 hx = xr[m], hy = yr[m];
                    float cy[2] = {diff(e.x, em, idy), diff(e.y, e.x, idy)};
                    float cx[2] = {diff(e.x, eu.x, idx_), diff(e.y, eu.y, idx_)};
                    float* hxp = &hx.x;
                    float* hyp = &hy.x;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const unsigned f = fl2[2 * m + h];
                        const unsigned qx = (f >> 8) & 255u, qy = (f >> 16) & 255u;
                        if ((f & 1u) && qy != 255u) cy[h] = cpml_d(cy[h], sb[qy], sa[qy], sk[qy], qXY[idx + h]);
                        if ((f & 2u) && qx != 255u) cx[h] = cpml_d(cx[h], sb[qx], sa[qx], sk[qx], qYX[idx + h]);
                        hxp[h] = (f & 1u) ? h_minus(hxp[h], cy[h], da, db) : hxp[h];
                        hyp[h] = (f & 2u) ? h_plus(hyp[h], cx[h], da, db) : hyp[h];
                    }
                    xr[m] = hx;
                    yr[m] = hy;
                    *reinterpret_cast<float2*>(sX + idx) = hx;
                    *reinterpret_cast<float2*>(sY + idx) = hy;
                }
                __syncthreads();
#pragma unroll
                for (int m = 0; m < MP; ++m) {
                    const int q = tid + m * BNT;
                    if (q >= NP) continue;
                    const int idx = pidx[m];
                    const float2 hx = xr[m], hy = yr[m];
                    const float2 hyd = *reinterpret_cast<const float2*>(sY + idx + RY);
                    const float hxn = sX[idx + 2];
                    float2 e = er[m];
                    float c1[2] = {diff(hyd.x, hy.x, idx_), diff(hyd.y, hy.y, idx_)};
                    float c2[2] = {diff(hx.y, hx.x, idy), diff(hxn, hx.y, idy)};
                    float* ep = &e.x;
                    const float cbv[2] = {cb2[m].x, cb2[m].y};
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const unsigned f = fl2[2 * m + h];
                        const unsigned qx = (f >> 8) & 255u, qy = (f >> 16) & 255u;
                        if ((f & 4u) && qx != 255u) c1[h] = cpml_d(c1[h], sb[qx], sa[qx], sk[qx], qZX[idx + h]);
                        if ((f & 4u) && qy != 255u) c2[h] = cpml_d(c2[h], sb[qy], sa[qy], sk[qy], qZY[idx + h]);
                        ep[h] = (f & 4u) ? __fmaf_rn(cbv[h], __fsub_rn(c1[h], c2[h]), ep[h]) : ep[h];
                        if (SPEC && (f & 4u) && (f & 48u) && P.live) {
                            // the soft source at t_{n+1}, then the port samples (split_e2 order)
                            const int gi = gx0 + idx / RY, gj = gy0 + (idx + h - (idx / RY) * RY);
                            if (f & 16u) ep[h] = __fadd_rn(ep[h], static_cast<float>(P.w[sI.w_off + (gj - sI.src_y0)] * amp));
                            if ((f & 32u) && P.ring)
                                for (int q2 = 0; q2 < sI.nport; ++q2)
                                    if (gi == sI.mx[q2] && (unsigned)(gj - sI.my0[q2]) < (unsigned)sI.mn[q2])
                                        P.ring[(int64_t)(P.row0 + s) * P.npts + sI.mpt[q2] + (gj - sI.my0[q2])] = ep[h];
                        }
                    }
                    er[m] = e;
                    *reinterpret_cast<float2*>(sE + idx) = e;
                }
                __syncthreads();
            }
            float chk = 0.f;
#pragma unroll
            for (int m = 0; m < MP; ++m) {
                const int q = tid + m * BNT;
                if (q >= NP) continue;
                const int idx = pidx[m];
                const int gi = gx0 + idx / RY;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const unsigned f = fl2[2 * m + h];
                    if (!(f & 8u)) continue;
                    const int gj = gy0 + (idx + h - (idx / RY) * RY);
                    const int64_t o = (int64_t)gi * pitch + gj;
                    chk += h ? er[m].y : er[m].x;
                    fout[o] = h ? er[m].y : er[m].x;
                    fout[nxp + o] = h ? xr[m].y : xr[m].x;
                    fout[2 * nxp + o] = h ? yr[m].y : yr[m].x;
                    const unsigned qx = (f >> 8) & 255u, qy = (f >> 16) & 255u;
                    if (qx != 255u) {
                        P.psi_out[pyx + (int64_t)qx * pitch + gj] = qYX[idx + h];
                        P.psi_out[pzx + (int64_t)qx * pitch + gj] = qZX[idx + h];
                    }
                    if (qy != 255u) {
                        P.psi_out[pxy + (int64_t)gi * (2 * t) + qy] = qXY[idx + h];
                        P.psi_out[pzy + (int64_t)gi * (2 * t) + qy] = qZY[idx + h];
                    }
                }
            }
            flag_nonfinite(P, it.x, chk);
            continue;
        }
    }
}

__global__ void batch_advance(long long* step, int n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *step += n;
}

struct Variant {
    int tx, ty, k, k1;  // tile, steps per pass, index of the K=1 sibling
    const void* fn[3];  // [0]: fast-path items, [1]: edge / CPML items, [2]: source / port items
    size_t smem[3];
};

#define PC_BV(TX, TY, K, K1)                                                                          \
    {TX,                                                                                              \
     TY,                                                                                              \
     K,                                                                                               \
     K1,                                                                                              \
     {reinterpret_cast<const void*>(&batch2d_pass<TX, TY, K, true, false>),                          \
      reinterpret_cast<const void*>(&batch2d_pass<TX, TY, K, false, false>),                         \
      reinterpret_cast<const void*>(&batch2d_pass<TX, TY, K, false, true>)},                          \
     {BShape<TX, TY, K>::SMEM_FAST, BShape<TX, TY, K>::SMEM, BShape<TX, TY, K>::SMEM}}
const Variant kVariants[] = {
    PC_BV(32, 64, 1, 0),  PC_BV(32, 64, 2, 0),  PC_BV(32, 64, 4, 0),  PC_BV(32, 64, 8, 0),
    PC_BV(16, 128, 1, 4), PC_BV(16, 128, 2, 4), PC_BV(16, 128, 4, 4), PC_BV(64, 64, 1, 7),
    PC_BV(64, 64, 2, 7),  PC_BV(64, 64, 4, 7),
    // smaller tiles: more CTAs for batches of few or small instances (a single
    // 500 x 250 grid is 64 tiles of 32 x 64 for 152 SMs)
    PC_BV(32, 32, 1, 10), PC_BV(32, 32, 2, 10), PC_BV(32, 32, 4, 10),
};
#undef PC_BV
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

}  // namespace
}  // namespace pc

using namespace pc;

struct pc_batch {
    int ninst = 0;
    int t = 0;
    double dx = 0, dy = 0, dt = 0, db_s = 0;
    std::vector<pc_batch_instance> desc;
    std::vector<BInst> inst;
    pc_batch_layout lay{};
    BInst* d_inst = nullptr;
    float* d_slab = nullptr;
    double* d_w = nullptr;
    double* d_amps = nullptr;
    int namps = 0;
    long long* d_step = nullptr;
    unsigned* d_status = nullptr;
    unsigned* d_inst_status = nullptr;  // [ninst]
    float* set[2] = {nullptr, nullptr};
    float* cb = nullptr;
    float* psi[2] = {nullptr, nullptr};
    bool bound = false, have_slab = false;
    int cur = 0;
    // DFT ports
    bool have_dft = false;
    DftMonitor dft{};
    int dft_rows = 0;
    // schedule
    int variant = 1;
    int graph_steps = 80;
    int item_variant = -1;
    int4* d_items = nullptr;  // fast-path items, then edge / CPML items, then source / port items
    int nitems = 0;
    int nfast = 0, ngen = 0;  // fast items, then edge / CPML ones, then source / port ones
    int items_cap = 0;
    int grid[kNumVariants][3] = {};
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_key[2][2] = {{-1, -1}, {-1, -1}};  // (variant, graph_steps) the graph was captured for
    int graph_nodes[2] = {0, 0};
    long long steps_done = 0;
    long long launches = 0;
};

namespace pc {
namespace {

int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

void drop_graphs(pc_batch* b) {
    for (int q = 0; q < 2; ++q) {
        if (b->graph[q]) cudaGraphExecDestroy(b->graph[q]);
        b->graph[q] = nullptr;
        b->graph_key[q][0] = b->graph_key[q][1] = -1;
    }
}

// (instance, tile) items for a variant's tile shape, LPT-sorted by estimated cost
int build_items(pc_batch* b, int v) {
    if (b->item_variant == v) return PC_OK;
    const Variant& V = kVariants[v];
    std::vector<int4> items;
    std::vector<float> cost;
    const int t = b->t, K = V.k;
    for (int n = 0; n < b->ninst; ++n) {
        const int nx = b->inst[n].nx, ny = b->inst[n].ny;
        for (int x0 = 0; x0 < nx; x0 += V.tx)
            for (int y0 = 0; y0 < ny; y0 += V.ty) {
                const int ax0 = x0 - K, ax1 = x0 + V.tx + K, ay0 = y0 - K, ay1 = y0 + V.ty + K;
                // bit 0: the region (with its halo) reaches the CPML or the instance edge
                // bit 1: it holds source or port cells (own class: the source and
                // port-sample code)
                const bool cp = ax0 < t || ax1 > nx - t || ay0 < t || ay1 > ny - t || ax0 < 0 || ay0 < 0 ||
                                ax1 > nx || ay1 > ny;
                const pc_batch_instance& d = b->desc[n];
                bool special = d.src_n > 0 && d.src_x >= ax0 && d.src_x < ax1 && d.src_y0 < ay1 &&
                               d.src_y0 + d.src_n > ay0;
                for (int q = 0; q < d.nport; ++q)
                    special = special || (d.port_x[q] >= ax0 && d.port_x[q] < ax1 && d.port_y0[q] < ay1 &&
                                          d.port_y0[q] + d.port_n[q] > ay0);
                items.push_back(make_int4(n, x0, y0, (cp ? 1 : 0) | (special ? 2 : 0)));
                const int cx = std::min(nx, x0 + V.tx) - x0, cy = std::min(ny, y0 + V.ty) - y0;
                cost.push_back((float)(cx * cy) * (cp ? 1.5f : 1.0f) + 0.25f * V.tx * V.ty);
            }
    }
    if (b->d_items) drop_graphs(b);  // captured graphs hold the previous table
    std::vector<int> ord(items.size());
    std::iota(ord.begin(), ord.end(), 0);
    // fast-path items first, then the edge / CPML ones without and then those with
    // source or port cells; each class longest first
    auto cls = [&](int a) { return (items[a].w & 2) ? 2 : ((items[a].w & 1) ? 1 : 0); };
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) {
        if (cls(a) != cls(c)) return cls(a) < cls(c);
        return cost[a] > cost[c];
    });
    std::vector<int4> sorted(items.size());
    int nfast = 0, ngen = 0;
    for (size_t q = 0; q < ord.size(); ++q) {
        sorted[q] = items[ord[q]];
        nfast += cls(ord[q]) == 0 ? 1 : 0;
        ngen += cls(ord[q]) == 1 ? 1 : 0;
    }
    if ((int)sorted.size() > b->items_cap) {
        cudaFree(b->d_items);
        b->d_items = nullptr;
        b->items_cap = 0;
        PC_CUDA_CHECK(cudaMalloc(&b->d_items, sorted.size() * sizeof(int4)));
        b->items_cap = (int)sorted.size();
    }
    PC_CUDA_CHECK(cudaMemcpy(b->d_items, sorted.data(), sorted.size() * sizeof(int4), cudaMemcpyHostToDevice));
    b->nitems = (int)sorted.size();
    b->nfast = nfast;
    b->ngen = ngen;
    b->item_variant = v;
    return PC_OK;
}

int grid_for(pc_batch* b, int v, int path) {
    if (b->grid[v][path] > 0) return b->grid[v][path];
    int dev = 0, nsm = 0, occ = 0;
    const Variant& V = kVariants[v];
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaFuncSetAttribute(V.fn[path], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)V.smem[path]) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, V.fn[path], BNT, V.smem[path]) != cudaSuccess)
        return -1;
    b->grid[v][path] = std::max(1, nsm * std::max(1, occ));
    return b->grid[v][path];
}

// A pass reads the current set and writes the other one, so a dry pass (live = 0)
// never changes the current state.
BPass make_pass(pc_batch* b, int s_off, int row0, bool live) {
    BPass P{};
    P.inst = b->d_inst;
    P.items = b->d_items;
    P.nitems = b->nitems;
    const int in = b->cur, out = b->cur ^ 1;
    P.fin = b->set[in];
    P.fout = b->set[out];
    P.cb = b->cb;
    P.psi_in = b->psi[in] ? b->psi[in] : b->psi[0];
    P.psi_out = b->psi[out] ? b->psi[out] : b->psi[0];
    P.slab = b->d_slab;
    P.t = b->t;
    P.inv_dx = (float)(1.0 / b->dx);
    P.inv_dy = (float)(1.0 / b->dy);
    P.da = 1.0f;
    P.db = (float)b->db_s;
    P.amps = b->d_amps;
    P.namps = b->namps;
    P.step = b->d_step;
    P.s_off = s_off;
    P.row0 = row0;
    P.ring = b->have_dft ? b->dft.d_ring : nullptr;
    P.npts = b->have_dft ? b->dft.npts : 0;
    P.w = b->d_w;
    P.live = live ? 1 : 0;
    P.status = b->d_status;
    P.inst_status = b->d_inst_status;
    return P;
}

// One pass = the fast-path items' kernel, then the edge / CPML items' kernel, then
// the source / port items' kernel; returns the number of kernels launched (or a
// negative error).
int launch_pass(pc_batch* b, int v, const BPass& P0, cudaStream_t s) {
    int launched = 0;
    for (int path = 0; path < 3; ++path) {
        BPass P = P0;
        const int first[3] = {0, b->nfast, b->nfast + b->ngen};
        P.items = P0.items + first[path];
        P.nitems = path == 2 ? P0.nitems - first[2] : first[path + 1] - first[path];
        if (P.nitems <= 0) continue;
        const int g = grid_for(b, v, path);
        if (g <= 0) return PC_ERR_CUDA;
        const int grid = std::min(g, P.nitems);
        void* args[] = {&P};
        PC_CUDA_CHECK(cudaLaunchKernel(kVariants[v].fn[path], dim3(grid), dim3(BNT), args, kVariants[v].smem[path], s));
        ++b->launches;
        ++launched;
    }
    return launched;
}

// One chunk of eager passes of variant v covering `steps` steps starting at ring row
// b->dft_rows; flushes the DFT ring whenever it fills and advances the step counter.
int run_passes(pc_batch* b, int v, int steps, cudaStream_t s, int* nodes) {
    const int K = kVariants[v].k;
    int done = 0;
    while (done < steps) {
        int vv = v, k = K;
        if (steps - done < K || (b->have_dft && b->dft_rows + K > RING_T)) {
            vv = kVariants[v].k1;
            k = 1;
        }
        // the K=1 sibling reuses the table of v (same tiles; halo flags computed for K >= 1)
        BPass P = make_pass(b, done, b->dft_rows, true);
        int rc = launch_pass(b, vv, P, s);
        if (rc < 0) return rc;
        *nodes += rc;
        b->cur ^= 1;
        done += k;
        if (b->have_dft) {
            b->dft_rows += k;
            if (b->dft_rows == RING_T) {
                rc = launch_dft_flush_rows(b->dft, RING_T, s);
                if (rc) return rc;
                b->launches += 2;
                *nodes += 2;
                b->dft_rows = 0;
            }
        }
    }
    batch_advance<<<1, 32, 0, s>>>(b->d_step, steps);
    PC_CUDA_CHECK(cudaGetLastError());
    ++b->launches;
    ++*nodes;
    return PC_OK;
}

int ensure_graph(pc_batch* b) {
    const int q = b->cur;
    if (b->graph[q] && b->graph_key[q][0] == b->variant && b->graph_key[q][1] == b->graph_steps) return PC_OK;
    if (b->graph[q]) {
        cudaGraphExecDestroy(b->graph[q]);
        b->graph[q] = nullptr;
    }
    if (!b->cap_stream) PC_CUDA_CHECK(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
    for (int path = 0; path < 2; ++path)
        if (grid_for(b, b->variant, path) <= 0 || grid_for(b, kVariants[b->variant].k1, path) <= 0)
            return PC_ERR_CUDA;
    const int cur0 = b->cur, rows0 = b->dft_rows;
    const long long launches0 = b->launches;
    int nodes = 0;
    cudaGraph_t gr = nullptr;
    PC_CUDA_CHECK(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
    int rc = run_passes(b, b->variant, b->graph_steps, b->cap_stream, &nodes);
    cudaError_t e = cudaStreamEndCapture(b->cap_stream, &gr);
    b->cur = cur0;
    b->dft_rows = rows0;
    b->launches = launches0;
    if (rc) {
        if (gr) cudaGraphDestroy(gr);
        return rc;
    }
    PC_CUDA_CHECK(e);
    e = cudaGraphInstantiate(&b->graph[q], gr, 0);
    cudaGraphDestroy(gr);
    PC_CUDA_CHECK(e);
    b->graph_key[q][0] = b->variant;
    b->graph_key[q][1] = b->graph_steps;
    b->graph_nodes[q] = nodes;
    return PC_OK;
}

bool graph_ok(const pc_batch* b) {
    const int K = kVariants[b->variant].k;
    return b->graph_steps > 0 && b->graph_steps % RING_T == 0 && (b->graph_steps / K) % 2 == 0;
}

}  // namespace
}  // namespace pc

extern "C" {

int pc_batch_create(int32_t ninst, const pc_batch_instance* desc, int32_t cpml_t, double dx, double dy, double dt,
                    double db_s, pc_batch** out, pc_batch_layout* lay) {
    if (!out || !lay || ninst <= 0 || !desc || cpml_t < 0 || cpml_t > 100 || !(dx > 0) || !(dy > 0) || !(dt > 0))
        return PC_ERR_INVALID;
    *out = nullptr;
    pc_batch* b = new pc_batch();
    b->ninst = ninst;
    b->t = cpml_t;
    b->dx = dx;
    b->dy = dy;
    b->dt = dt;
    b->db_s = db_s;
    b->desc.assign(desc, desc + ninst);
    int64_t foff = 0, coff = 0, poff = 0, woff = 0, pts = 0;
    for (int n = 0; n < ninst; ++n) {
        const pc_batch_instance& d = desc[n];
        if (d.nx < 2 * cpml_t + 4 || d.ny < 2 * cpml_t + 4 || d.nx > (1 << 20) || d.ny > (1 << 20) || d.nport < 0 ||
            d.nport > 4 || d.src_n < 0 || d.src_x < 0 || d.src_x >= d.nx - 1 || d.src_y0 < 0 ||
            d.src_y0 + d.src_n > d.ny - 1) {
            delete b;
            return PC_ERR_INVALID;
        }
        BInst I{};
        I.nx = d.nx;
        I.ny = d.ny;
        I.pitch = (int)round_up(d.ny, 32);
        I.src_x = d.src_x;
        I.src_y0 = d.src_y0;
        I.src_n = d.src_n;
        I.nport = d.nport;
        I.f_off = foff;
        I.c_off = coff;
        I.p_off = poff;
        I.w_off = woff;
        for (int q = 0; q < 4; ++q) I.mx[q] = I.my0[q] = I.mn[q] = I.mpt[q] = 0;
        for (int q = 0; q < d.nport; ++q) {
            if (d.port_x[q] < 0 || d.port_x[q] >= d.nx - 1 || d.port_y0[q] < 0 || d.port_n[q] <= 0 ||
                d.port_y0[q] + d.port_n[q] > d.ny - 1) {
                delete b;
                return PC_ERR_INVALID;
            }
            I.mx[q] = d.port_x[q];
            I.my0[q] = d.port_y0[q];
            I.mn[q] = d.port_n[q];
            I.mpt[q] = (int)pts;
            pts += d.port_n[q];
        }
        const int64_t plane = (int64_t)d.nx * I.pitch;
        foff += 3 * plane;
        coff += plane;
        poff += 4 * (int64_t)cpml_t * (I.pitch + d.nx);
        woff += d.src_n;
        b->inst.push_back(I);
    }
    b->lay.field_elems = foff;
    b->lay.coef_elems = coff;
    b->lay.psi_elems = std::max<int64_t>(poff, 1);
    b->lay.weight_elems = woff;
    b->lay.dft_points = pts;
    *lay = b->lay;
    bool ok = cudaMalloc(&b->d_inst, ninst * sizeof(BInst)) == cudaSuccess &&
              cudaMalloc(&b->d_step, sizeof(long long)) == cudaSuccess &&
              cudaMalloc(&b->d_status, sizeof(unsigned)) == cudaSuccess &&
              cudaMalloc(&b->d_inst_status, ninst * sizeof(unsigned)) == cudaSuccess &&
              cudaMalloc(&b->d_w, std::max<int64_t>(woff, 1) * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&b->d_slab, std::max(1, 6 * cpml_t) * sizeof(float)) == cudaSuccess;
    ok = ok && cudaMemcpy(b->d_inst, b->inst.data(), ninst * sizeof(BInst), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(b->d_step, 0, sizeof(long long)) == cudaSuccess &&
         cudaMemset(b->d_status, 0, sizeof(unsigned)) == cudaSuccess &&
         cudaMemset(b->d_inst_status, 0, ninst * sizeof(unsigned)) == cudaSuccess &&
         cudaMemset(b->d_w, 0, std::max<int64_t>(woff, 1) * sizeof(double)) == cudaSuccess;
    if (!ok) {
        pc_batch_destroy(b);
        return PC_ERR_CUDA;
    }
    b->have_slab = cpml_t == 0;
    *out = b;
    return PC_OK;
}

int pc_batch_instance_offsets(const pc_batch* b, int32_t i, int64_t out[5]) {
    if (!b || !out || i < 0 || i >= b->ninst) return PC_ERR_INVALID;
    const BInst& I = b->inst[i];
    out[0] = I.f_off;
    out[1] = I.pitch;
    out[2] = I.c_off;
    out[3] = I.w_off;
    out[4] = I.nport ? I.mpt[0] : -1;
    return PC_OK;
}

int pc_batch_bind(pc_batch* b, void* d_set0, void* d_set1, void* d_cb, void* d_psi0, void* d_psi1) {
    if (!b || !d_set0 || !d_set1 || !d_cb || d_set0 == d_set1) return PC_ERR_INVALID;
    if (b->t > 0 && (!d_psi0 || !d_psi1 || d_psi0 == d_psi1)) return PC_ERR_INVALID;
    b->set[0] = static_cast<float*>(d_set0);
    b->set[1] = static_cast<float*>(d_set1);
    b->cb = static_cast<float*>(d_cb);
    b->psi[0] = static_cast<float*>(d_psi0);
    b->psi[1] = static_cast<float*>(d_psi1);
    b->cur = 0;
    b->bound = true;
    drop_graphs(b);
    return PC_OK;
}

int pc_batch_build_coefficients(pc_batch* b, int32_t i, const double* d_eps, double eps0, void* stream) {
    if (!b || !b->bound || i < 0 || i >= b->ninst || !d_eps || !(eps0 > 0)) return PC_ERR_INVALID;
    const BInst& I = b->inst[i];
    pc_grid_desc g{};
    g.ndim = 2;
    g.nx = I.nx;
    g.ny = I.ny;
    g.nz = 1;
    g.pitch = I.pitch;
    g.precision = 4;
    g.dt = b->dt;
    void* cb[3] = {nullptr, nullptr, b->cb + I.c_off};
    int64_t l = 0;
    int rc = launch_build_coefficients(g, d_eps, nullptr, nullptr, nullptr, eps0, 1.0, nullptr, cb, nullptr, nullptr,
                                       (cudaStream_t)stream, &l);
    b->launches += l;
    return rc;
}

int pc_batch_set_cpml(pc_batch* b, const double* bcoef, const double* acoef, const double* kappa) {
    if (!b || b->t <= 0 || !bcoef || !acoef || !kappa) return PC_ERR_INVALID;
    const int t2 = 2 * b->t;
    std::vector<float> h(3 * t2);
    for (int q = 0; q < t2; ++q) {
        if (!(kappa[q] > 0)) return PC_ERR_INVALID;
        h[q] = (float)bcoef[q];
        h[t2 + q] = (float)acoef[q];
        h[2 * t2 + q] = (float)(1.0 / kappa[q]);
    }
    PC_CUDA_CHECK(cudaMemcpy(b->d_slab, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    b->have_slab = true;
    return PC_OK;
}

int pc_batch_set_sources(pc_batch* b, const double* weights, const double* amps, int32_t namps) {
    if (!b || namps < 0 || (namps > 0 && !amps) || (b->lay.weight_elems > 0 && !weights)) return PC_ERR_INVALID;
    // passes already queued (on any stream) may still read the tables being replaced
    if (b->steps_done > 0) PC_CUDA_CHECK(cudaDeviceSynchronize());
    if (namps != b->namps) drop_graphs(b);  // captured passes hold the table's address and length
    if (b->lay.weight_elems > 0)
        PC_CUDA_CHECK(cudaMemcpy(b->d_w, weights, b->lay.weight_elems * sizeof(double), cudaMemcpyHostToDevice));
    if (namps > b->namps || !b->d_amps) {
        cudaFree(b->d_amps);
        b->d_amps = nullptr;
        PC_CUDA_CHECK(cudaMalloc(&b->d_amps, std::max(1, namps) * sizeof(double)));
    }
    if (namps > 0) PC_CUDA_CHECK(cudaMemcpy(b->d_amps, amps, namps * sizeof(double), cudaMemcpyHostToDevice));
    b->namps = namps;
    return PC_OK;
}

int pc_batch_set_dft(pc_batch* b, const double* omega, int32_t nf, double t0, void* d_acc) {
    if (!b || b->have_dft || b->lay.dft_points <= 0 || b->lay.dft_points > INT32_MAX) return PC_ERR_INVALID;
    std::vector<int64_t> offs(b->lay.dft_points);
    for (const BInst& I : b->inst)
        for (int q = 0; q < I.nport; ++q)
            for (int y = 0; y < I.mn[q]; ++y)
                offs[I.mpt[q] + y] = I.f_off + (int64_t)I.mx[q] * I.pitch + I.my0[q] + y;
    const int rc = dft_monitor_init(b->dft, 2, offs.data(), (int)offs.size(), omega, nf, b->dt, t0, d_acc,
                                    b->lay.field_elems);
    if (rc) return rc;
    b->have_dft = true;
    b->dft_rows = 0;
    drop_graphs(b);
    return PC_OK;
}

int pc_batch_num_variants(void) { return kNumVariants; }

int pc_batch_variant_info(int32_t v, int32_t out[3]) {
    if (v < 0 || v >= kNumVariants || !out) return PC_ERR_INVALID;
    out[0] = kVariants[v].tx;
    out[1] = kVariants[v].ty;
    out[2] = kVariants[v].k;
    return PC_OK;
}

int pc_batch_set_tuning(pc_batch* b, int32_t variant, int32_t graph_steps) {
    if (!b || variant < 0 || variant >= kNumVariants || graph_steps < 0) return PC_ERR_INVALID;
    const int old_v = b->variant, old_g = b->graph_steps;
    b->variant = variant;
    b->graph_steps = graph_steps;
    if (graph_steps > 0 && !graph_ok(b)) {
        b->variant = old_v;
        b->graph_steps = old_g;
        return PC_ERR_INVALID;
    }
    return PC_OK;
}

int pc_batch_get_tuning(const pc_batch* b, int32_t* variant, int32_t* graph_steps) {
    if (!b || !variant || !graph_steps) return PC_ERR_INVALID;
    *variant = b->variant;
    *graph_steps = b->graph_steps;
    return PC_OK;
}

int pc_batch_autotune(pc_batch* b, int32_t passes, float* ms_per_step, void* stream) {
    if (!b || !b->bound || passes <= 0 || (b->t > 0 && !b->have_slab)) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    PC_CUDA_CHECK(cudaEventCreate(&e0));
    PC_CUDA_CHECK(cudaEventCreate(&e1));
    float best = 1e30f;
    int bestv = b->variant;
    for (int v = 0; v < kNumVariants; ++v) {
        int rc = build_items(b, v);
        if (rc) return rc;
        BPass P = make_pass(b, 0, 0, false);
        rc = launch_pass(b, v, P, s);  // warm-up
        if (rc < 0) return rc;
        PC_CUDA_CHECK(cudaEventRecord(e0, s));
        for (int q = 0; q < passes; ++q) {
            rc = launch_pass(b, v, P, s);
            if (rc < 0) return rc;
        }
        PC_CUDA_CHECK(cudaEventRecord(e1, s));
        PC_CUDA_CHECK(cudaEventSynchronize(e1));
        float ms = 0.f;
        PC_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
        const float per_step = ms / (passes * kVariants[v].k);
        if (ms_per_step) ms_per_step[v] = per_step;
        if (per_step < best) {
            best = per_step;
            bestv = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->variant = bestv;
    if (b->graph_steps > 0 && !graph_ok(b)) b->graph_steps = 16 * 2 * kVariants[bestv].k;
    return PC_OK;
}

int pc_batch_step(pc_batch* b, int32_t nsteps, void* stream) {
    if (!b || nsteps < 0) return PC_ERR_INVALID;
    if (!b->bound || (b->t > 0 && !b->have_slab)) return PC_ERR_STATE;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = build_items(b, b->variant);
    if (rc) return rc;
    const bool use_graph = b->graph_steps > 0 && graph_ok(b);
    while (nsteps > 0) {
        if (use_graph && b->dft_rows == 0 && nsteps >= b->graph_steps) {
            rc = ensure_graph(b);
            if (rc) return rc;
            PC_CUDA_CHECK(cudaGraphLaunch(b->graph[b->cur], s));
            b->launches += b->graph_nodes[b->cur];
            b->steps_done += b->graph_steps;
            nsteps -= b->graph_steps;
            continue;  // an even number of passes: the current set is unchanged
        }
        // eager passes up to the next ring boundary (or the end)
        int chunk = nsteps;
        if (b->have_dft) chunk = std::min(chunk, RING_T - b->dft_rows);
        int nodes = 0;
        rc = run_passes(b, b->variant, chunk, s, &nodes);
        if (rc) return rc;
        b->steps_done += chunk;
        nsteps -= chunk;
    }
    return PC_OK;
}

int pc_batch_dft_flush(pc_batch* b, void* stream) {
    if (!b) return PC_ERR_INVALID;
    if (!b->have_dft || b->dft_rows == 0) return PC_OK;
    const int rc = launch_dft_flush_rows(b->dft, b->dft_rows, (cudaStream_t)stream);
    if (rc) return rc;
    b->launches += 2;
    b->dft_rows = 0;
    return PC_OK;
}

int pc_batch_current_set(const pc_batch* b) { return b ? b->cur : PC_ERR_INVALID; }

int pc_batch_status(pc_batch* b, uint32_t* flags, void* stream) {
    if (!b || !flags) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned v = 0;
    PC_CUDA_CHECK(cudaMemcpyAsync(&v, b->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    PC_CUDA_CHECK(cudaStreamSynchronize(s));
    *flags = v;
    return PC_OK;
}

int pc_batch_instance_status(pc_batch* b, uint32_t* flags, void* stream) {
    if (!b || !flags) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    static_assert(sizeof(unsigned) == sizeof(uint32_t), "status word size");
    PC_CUDA_CHECK(cudaMemcpyAsync(flags, b->d_inst_status, b->ninst * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    PC_CUDA_CHECK(cudaMemsetAsync(b->d_inst_status, 0, b->ninst * sizeof(unsigned), s));
    PC_CUDA_CHECK(cudaStreamSynchronize(s));
    return PC_OK;
}

int64_t pc_batch_launch_count(const pc_batch* b) { return b ? b->launches : PC_ERR_INVALID; }

int64_t pc_batch_steps_done(const pc_batch* b) { return b ? b->steps_done : PC_ERR_INVALID; }

void pc_batch_destroy(pc_batch* b) {
    if (!b) return;
    drop_graphs(b);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    if (b->have_dft) dft_monitor_free(b->dft);
    cudaFree(b->d_inst);
    cudaFree(b->d_slab);
    cudaFree(b->d_w);
    cudaFree(b->d_amps);
    cudaFree(b->d_step);
    cudaFree(b->d_status);
    cudaFree(b->d_inst_status);
    cudaFree(b->d_items);
    delete b;
}

}  // extern "C"
