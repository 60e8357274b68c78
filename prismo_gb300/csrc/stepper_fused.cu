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
#include <cuda.h>

#include <algorithm>

#include "pc_internal.cuh"
#include "stencil_common.cuh"
#include "tma.cuh"

namespace pc {

struct FusedMaps {
    CUtensorMap e[3];
    CUtensorMap h[3];
    CUtensorMap cb[3];
};

namespace {

constexpr uint32_t kWaitLimit = 1u << 22;

template <typename T, int TY, int TZ>
struct FusedGeom {
    static constexpr int EW = TZ + 8;  // E box: k in [k0-4, k0+TZ+4)
    static constexpr int EH = TY + 2;  //        j in [j0-1, j0+TY+1)
    static constexpr int HW = TZ + 4;  // H box: k in [k0, k0+TZ+4)
    static constexpr int HH = TY + 1;  //        j in [j0, j0+TY+1)
    static constexpr int CW = TZ;      // Cb box: the tile
    static constexpr int CH = TY;
    static constexpr int align128(int b) { return (b + 127) / 128 * 128; }
    static constexpr int E_BOX = align128(EW * EH * (int)sizeof(T));
    static constexpr int H_BOX = align128(HW * HH * (int)sizeof(T));
    static constexpr int C_BOX = align128(CW * CH * (int)sizeof(T));
    static constexpr int STAGE = 3 * (E_BOX + H_BOX + C_BOX);
    static constexpr uint32_t TX_BYTES = 3u * (EW * EH + HW * HH + CW * CH) * sizeof(T);
    static constexpr int HN_PLANE = 3 * HH * HW;  // elements of one H^{n+1/2} plane (3 comps)
};

template <typename T, int TY, int TZ, int S>
constexpr int fused_smem_bytes() {
    using G = FusedGeom<T, TY, TZ>;
    return 128 + S * G::STAGE + 2 * G::HN_PLANE * (int)sizeof(T);
}

template <typename T, int AX>
__device__ __forceinline__ T cpml3w(const CpmlArgs<T>& p, int slot, const Idx3& q, T d, bool write) {
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
    const T psi = p.b[AX][idx] * p.psi_in[po] + p.a[AX][idx] * d;
    if (write) p.psi_out[po] = psi;
    return d * p.kinv[AX][idx] + psi;
}

template <typename T, int TY, int TZ, int S, bool CPML>
__global__ void __launch_bounds__(TY* TZ, 2)
    fused3(FieldArgs<T> a, CpmlArgs<T> pm, int cx, const __grid_constant__ FusedMaps maps) {
    using G = FusedGeom<T, TY, TZ>;
    constexpr int EW = G::EW, HW = G::HW, CW = G::CW;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    unsigned char* stages = smem + 128;
    T* sHn = reinterpret_cast<T*>(stages + S * G::STAGE);

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * TZ + tx;
    const int k0 = blockIdx.x * TZ, j0 = blockIdx.y * TY;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int ib = blockIdx.z * cx;
    const int ie = min(nx, ib + cx);
    const int L = ie - ib + 2;  // planes ib-1 .. ie
    const int64_t P = a.pitch;

    if (tid == 0) {
        for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
        for (int c = 0; c < 3; ++c) {
            prefetch_tmap(&maps.e[c]);
            prefetch_tmap(&maps.h[c]);
            prefetch_tmap(&maps.cb[c]);
        }
    }
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
            tma_load_3d(st + 3 * (G::E_BOX + G::H_BOX) + c * G::C_BOX, &maps.cb[c], k0, j0, pl, &bars[s]);
    };
    int issued = L < S ? L : S;
    if (tid == 0)
        for (int n = 0; n < issued; ++n) issue(n);

    auto Ebox = [&](int n, int c) {
        return reinterpret_cast<const T*>(stages + (n % S) * G::STAGE + c * G::E_BOX);
    };
    auto Hbox = [&](int n, int c) {
        return reinterpret_cast<const T*>(stages + (n % S) * G::STAGE + 3 * G::E_BOX + c * G::H_BOX);
    };
    auto Cbox = [&](int n, int c) {
        return reinterpret_cast<const T*>(stages + (n % S) * G::STAGE + 3 * (G::E_BOX + G::H_BOX) + c * G::C_BOX);
    };
    auto Hn = [&](int plane, int c) { return sHn + (plane & 1) * G::HN_PLANE + c * (G::HH * HW); };

    // H^{n+1/2} at (p, j0+jj, k0+kk) into shared memory; psi written only when own.
    auto h_point = [&](int n, int p, int jj, int kk, bool own) {
        const int j = j0 + jj, k = k0 + kk;
        const int ho = jj * HW + kk;
        const int ei = (jj + 1) * EW + (kk + 4);
        const T* Exc = Ebox(n, 0);
        const T* Eyc = Ebox(n, 1);
        const T* Ezc = Ebox(n, 2);
        const T* Eyp = Ebox(n - 1, 1);
        const T* Ezp = Ebox(n - 1, 2);
        T hx = Hbox(n, 0)[ho], hy = Hbox(n, 1)[ho], hz = Hbox(n, 2)[ho];
        const Idx3 q{p, j, k, nx, ny, nz, a.pitch};
        const int64_t o = ((int64_t)p * ny + j) * P + k;
        if (p < nx - 1 && j >= 1 && j <= ny - 2 && k >= 1 && k <= nz - 2) {
            T cy = (Ezc[ei] - Ezc[ei - EW]) * a.inv_dy;
            T cz = (Eyc[ei] - Eyc[ei - 1]) * a.inv_dz;
            if (CPML) {
                cy = cpml3w<T, 1>(pm, SY_HX, q, cy, own);
                cz = cpml3w<T, 2>(pm, SZ_HX, q, cz, own);
            }
            hx = hcoef(a.da[0], o, a.da_s) * hx - hcoef(a.db[0], o, a.db_s) * (cy - cz);
        }
        if (p >= 1 && p <= nx - 2 && j <= ny - 2 && k >= 1 && k <= nz - 2) {
            T cz = (Exc[ei] - Exc[ei - 1]) * a.inv_dz;
            T cx_ = (Ezc[ei] - Ezp[ei]) * a.inv_dx;
            if (CPML) {
                cz = cpml3w<T, 2>(pm, SZ_HY, q, cz, own);
                cx_ = cpml3w<T, 0>(pm, SX_HY, q, cx_, own);
            }
            hy = hcoef(a.da[1], o, a.da_s) * hy - hcoef(a.db[1], o, a.db_s) * (cz - cx_);
        }
        if (p >= 1 && p <= nx - 2 && j >= 1 && j <= ny - 2 && k <= nz - 2) {
            T cx_ = (Eyc[ei] - Eyp[ei]) * a.inv_dx;
            T cy = (Exc[ei] - Exc[ei - EW]) * a.inv_dy;
            if (CPML) {
                cx_ = cpml3w<T, 0>(pm, SX_HZ, q, cx_, own);
                cy = cpml3w<T, 1>(pm, SY_HZ, q, cy, own);
            }
            hz = hcoef(a.da[2], o, a.da_s) * hz - hcoef(a.db[2], o, a.db_s) * (cx_ - cy);
        }
        Hn(p, 0)[ho] = hx;
        Hn(p, 1)[ho] = hy;
        Hn(p, 2)[ho] = hz;
    };

    bool timed_out = false;
    int n = 0;
    for (; n < L; ++n) {
        const bool ok = mbar_wait_bounded(&bars[n % S], (uint32_t)((n / S) & 1), kWaitLimit);
        const int pc_ = ib - 1 + n;  // plane whose H^{n+1/2} is computed now
        if (n >= 1 && ok) {
            h_point(n, pc_, ty, tx, pc_ < ie);
            if (tid < TZ + 1)
                h_point(n, pc_, TY, tid, false);
            else if (tid < TZ + 1 + TY)
                h_point(n, pc_, tid - (TZ + 1), TZ, false);
        }
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        const int j = j0 + ty, k = k0 + tx;
        const bool inside = j < ny && k < nz;
        if (n >= 2) {
            // E^{n+1} at plane q = pc_ - 1, own point
            const int q = pc_ - 1;
            const int ei = (ty + 1) * EW + (tx + 4);
            const int hi = ty * HW + tx;
            const int ci = ty * CW + tx;
            const T* Hxq = Hn(q, 0);
            const T* Hyq = Hn(q, 1);
            const T* Hzq = Hn(q, 2);
            const T* Hyp = Hn(pc_, 1);
            const T* Hzp = Hn(pc_, 2);
            T ex = Ebox(n - 1, 0)[ei], ey = Ebox(n - 1, 1)[ei], ez = Ebox(n - 1, 2)[ei];
            const Idx3 qq{q, j, k, nx, ny, nz, a.pitch};
            const int64_t o = ((int64_t)q * ny + j) * P + k;
            if (j <= ny - 2 && k <= nz - 2) {
                T c1 = (Hzq[hi + HW] - Hzq[hi]) * a.inv_dy;
                T c2 = (Hyq[hi + 1] - Hyq[hi]) * a.inv_dz;
                if (CPML) {
                    c1 = cpml3w<T, 1>(pm, SY_EX, qq, c1, true);
                    c2 = cpml3w<T, 2>(pm, SZ_EX, qq, c2, true);
                }
                ex = ecoef(a.ca[0], o) * ex + Cbox(n - 1, 0)[ci] * (c1 - c2);
            }
            if (q <= nx - 2 && k <= nz - 2) {
                T c1 = (Hxq[hi + 1] - Hxq[hi]) * a.inv_dz;
                T c2 = (Hzp[hi] - Hzq[hi]) * a.inv_dx;
                if (CPML) {
                    c1 = cpml3w<T, 2>(pm, SZ_EY, qq, c1, true);
                    c2 = cpml3w<T, 0>(pm, SX_EY, qq, c2, true);
                }
                ey = ecoef(a.ca[1], o) * ey + Cbox(n - 1, 1)[ci] * (c1 - c2);
            }
            if (q <= nx - 2 && j <= ny - 2) {
                T c1 = (Hyp[hi] - Hyq[hi]) * a.inv_dx;
                T c2 = (Hxq[hi + HW] - Hxq[hi]) * a.inv_dy;
                if (CPML) {
                    c1 = cpml3w<T, 0>(pm, SX_EZ, qq, c1, true);
                    c2 = cpml3w<T, 1>(pm, SY_EZ, qq, c2, true);
                }
                ez = ecoef(a.ca[2], o) * ez + Cbox(n - 1, 2)[ci] * (c1 - c2);
            }
            if (inside) {
                a.Eout[0][o] = ex;
                a.Eout[1][o] = ey;
                a.Eout[2][o] = ez;
                if (!(isfinite(ex) && isfinite(ey) && isfinite(ez))) atomicOr(a.status, PC_STATUS_NONFINITE);
            }
        }
        if (n >= 1 && pc_ < ie && inside) {
            const int64_t o = ((int64_t)pc_ * ny + j) * P + k;
            const int hi = ty * HW + tx;
            a.Hout[0][o] = Hn(pc_, 0)[hi];
            a.Hout[1][o] = Hn(pc_, 1)[hi];
            a.Hout[2][o] = Hn(pc_, 2)[hi];
        }
        __syncthreads();
        if (n >= 1 && n - 1 + S < L) {
            if (tid == 0) issue(n - 1 + S);
            ++issued;
        }
    }
    if (timed_out) {
        if (tid == 0) atomicOr(a.status, PC_STATUS_TIMEOUT);
        // let every copy already in flight land before the CTA retires
        for (int m = n; m < issued; ++m) mbar_wait_bounded(&bars[m % S], (uint32_t)((m / S) & 1), kWaitLimit);
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
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? PC_OK : PC_ERR_CUDA;
}

struct FusedState {
    const void* key_f[2][6];
    const void* key_cb[3];
    FusedMaps maps[2];  // per input set
    bool ready = false;
};

// One cached set of maps per context (keyed by the buffer pointers).
FusedState* state_of(pc_ctx* c) {
    if (!c->fused_state) c->fused_state = new FusedState();
    return static_cast<FusedState*>(c->fused_state);
}

template <typename T, int TY, int TZ, int S>
int fused_t(pc_ctx* c, cudaStream_t s) {
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
                if (!rc) rc = make_map(&st->maps[set].cb[q], c->cb[q], g, G::CW, G::CH);
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
    constexpr int smem = fused_smem_bytes<T, TY, TZ, S>();
    static bool attr_set[2] = {false, false};
    auto kern_cp = fused3<T, TY, TZ, S, true>;
    auto kern_nc = fused3<T, TY, TZ, S, false>;
    if (!attr_set[sizeof(T) == 8]) {
        PC_CUDA_CHECK(cudaFuncSetAttribute(kern_cp, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        PC_CUDA_CHECK(cudaFuncSetAttribute(kern_nc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr_set[sizeof(T) == 8] = true;
    }
    int cx = c->fused_cx;
    if (cx <= 0) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
        if (sms <= 0) sms = 152;
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern_cp, TY * TZ, smem);
        if (per_sm <= 0) per_sm = 1;
        const int resident = sms * per_sm;
        const int tiles = ((g.nz + TZ - 1) / TZ) * ((g.ny + TY - 1) / TY);
        // cost model: waves x planes streamed per CTA (chunk + 2 pipeline planes)
        const int cands[] = {8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512};
        double best = 1e300;
        cx = g.nx;
        for (int cand : cands) {
            if (cand > g.nx) break;
            const int chunks = (g.nx + cand - 1) / cand;
            const double ctas = (double)tiles * chunks;
            const double waves = ctas / resident;
            const double cost = (waves < 1.0 ? 1.0 : waves) * (cand + 2);
            if (cost < best * 0.97) {
                best = cost;
                cx = cand;
            }
        }
        c->fused_cx = cx;
    }
    dim3 blk(TZ, TY);
    dim3 grd((g.nz + TZ - 1) / TZ, (g.ny + TY - 1) / TY, (g.nx + cx - 1) / cx);
    if (p.t > 0)
        kern_cp<<<grd, blk, smem, s>>>(a, p, cx, st->maps[in]);
    else
        kern_nc<<<grd, blk, smem, s>>>(a, p, cx, st->maps[in]);
    PC_CUDA_CHECK(cudaGetLastError());
    ++c->launches;
    c->cur = out;
    return PC_OK;
}

}  // namespace

int launch_fused_step(pc_ctx* c, cudaStream_t s) {
    if (c->g.ndim != 3) return launch_split_step(c, s);
    if (c->g.precision == 8) return fused_t<double, 8, 32, 3>(c, s);
    return fused_t<float, 8, 32, 6>(c, s);
}

void destroy_fused_state(pc_ctx* c) {
    delete static_cast<FusedState*>(c->fused_state);
    c->fused_state = nullptr;
}

}  // namespace pc
