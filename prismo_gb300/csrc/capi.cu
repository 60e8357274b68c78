// extern "C" entry points of libprismo_cuda.so (declared in include/prismo_cuda.h).
#include <stdlib.h>
#include <string.h>

#include <math.h>

#include <new>
#include <vector>

#include "pc_internal.cuh"

namespace pc {

PsiLayout psi_layout(const pc_grid_desc& g, int t) {
    PsiLayout L{};
    L.t = t;
    if (t <= 0) return L;
    const int64_t T2 = 2 * (int64_t)t;
    if (g.ndim == 3) {
        L.slot_elems[0] = T2 * g.ny * g.pitch;
        L.slot_elems[1] = (int64_t)g.nx * T2 * g.pitch;
        L.slot_elems[2] = (int64_t)g.nx * g.ny * T2;
    } else {
        L.slot_elems[0] = T2 * g.pitch;
        L.slot_elems[1] = (int64_t)g.nx * T2;
        L.slot_elems[2] = 0;
    }
    int64_t off = 0;
    for (int ax = 0; ax < 3; ++ax) {
        L.axis_base[ax] = off;
        off += 4 * L.slot_elems[ax];
    }
    L.total = off;
    return L;
}

int dft_monitor_init(DftMonitor& m, int comp, const int64_t* offsets, int npts, const double* omega, int nf, double dt,
                     double t0, void* d_acc, int64_t limit) {
    if (npts <= 0 || !offsets || !omega || nf <= 0 || !(dt > 0) || !d_acc) return PC_ERR_INVALID;
    for (int i = 0; i < npts; ++i)
        if (offsets[i] < 0 || offsets[i] >= limit) return PC_ERR_INVALID;
    m = DftMonitor{};
    m.plane_k = -1;
    m.comp = comp;
    m.npts = npts;
    m.nf = nf;
    m.T = 16;
    m.dt = dt;
    m.d_acc = static_cast<float4*>(d_acc);
    std::vector<double> st(2 * nf), rot(2 * nf);
    for (int f = 0; f < nf; ++f) {
        // phase of the first sample, t0 = t_{n+1} of the next step, and one-step rotation
        st[2 * f] = cos(-omega[f] * t0);
        st[2 * f + 1] = sin(-omega[f] * t0);
        rot[2 * f] = cos(-omega[f] * dt);
        rot[2 * f + 1] = sin(-omega[f] * dt);
    }
    bool ok = cudaMalloc(&m.d_off, npts * sizeof(int64_t)) == cudaSuccess &&
              cudaMalloc(&m.d_ring, (size_t)m.T * npts * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&m.d_table, (size_t)m.T * nf * sizeof(float2)) == cudaSuccess &&
              cudaMalloc(&m.d_state, nf * sizeof(double2)) == cudaSuccess &&
              cudaMalloc(&m.d_rot, nf * sizeof(double2)) == cudaSuccess;
    ok = ok && cudaMemcpy(m.d_off, offsets, npts * sizeof(int64_t), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(m.d_state, st.data(), nf * sizeof(double2), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(m.d_rot, rot.data(), nf * sizeof(double2), cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        dft_monitor_free(m);
        return PC_ERR_CUDA;
    }
    return PC_OK;
}

void dft_monitor_free(DftMonitor& m) {
    cudaFree(m.d_off);
    cudaFree(m.d_ring);
    cudaFree(m.d_table);
    cudaFree(m.d_state);
    cudaFree(m.d_rot);
    m.d_off = nullptr;
    m.d_ring = nullptr;
    m.d_table = nullptr;
    m.d_state = nullptr;
    m.d_rot = nullptr;
}

}  // namespace pc

using namespace pc;

static int validate(const pc_grid_desc* d) {
    if (!d) return PC_ERR_INVALID;
    if (d->ndim != 2 && d->ndim != 3) return PC_ERR_INVALID;
    if (d->precision != 4 && d->precision != 8) return PC_ERR_INVALID;
    if (d->mode != PC_MODE_CORRECTED && d->mode != PC_MODE_LEGACY) return PC_ERR_INVALID;
    if (d->sched < PC_SCHED_AUTO || d->sched > PC_SCHED_FUSED) return PC_ERR_INVALID;
    if (d->nx < 3 || d->ny < 3) return PC_ERR_INVALID;
    if (d->ndim == 3 && d->nz < 3) return PC_ERR_INVALID;
    if (d->ndim == 2 && d->nz != 1) return PC_ERR_INVALID;
    const int fast = d->ndim == 3 ? d->nz : d->ny;
    if (d->pitch < fast || (d->pitch % 32) != 0) return PC_ERR_INVALID;
    if (!(d->dt > 0) || !(d->dx > 0) || !(d->dy > 0)) return PC_ERR_INVALID;
    if (d->ndim == 3 && !(d->dz > 0)) return PC_ERR_INVALID;
    if ((int64_t)d->nx * d->ny * d->pitch > ((int64_t)1 << 40)) return PC_ERR_INVALID;
    return PC_OK;
}

extern "C" {

int pc_version(void) { return 100; }

int pc_create(const pc_grid_desc* desc, pc_ctx** out) {
    if (!out) return PC_ERR_INVALID;
    *out = nullptr;
    int rc = validate(desc);
    if (rc) return rc;
    pc_ctx* c = new (std::nothrow) pc_ctx();
    if (!c) return PC_ERR_INVALID;
    c->g = *desc;
    if (c->g.sched == PC_SCHED_AUTO)
        c->g.sched = (c->g.ndim == 3 && c->g.mode == PC_MODE_CORRECTED) ? PC_SCHED_FUSED : PC_SCHED_SPLIT;
    if (c->g.mode == PC_MODE_LEGACY || c->g.ndim == 2) c->g.sched = PC_SCHED_SPLIT;
    c->da_s = 1.0;
    c->db_s = 0.0;
    c->gen = 1;
    c->warm_gen = 0;
    c->graph_steps = 64;
    c->fused_split = 2;
    c->fused_unified = 1;
    c->fused_extras = 1;
    c->ts_k = 2;  // temporally blocked stepper where it applies (pc_set_tuning)
    c->ts_order = 2;
    c->graph_gen[0] = c->graph_gen[1] = 0;
    if (cudaMalloc(&c->d_status, 2 * sizeof(uint32_t)) != cudaSuccess) {
        delete c;
        return PC_ERR_CUDA;
    }
    c->d_legacy_flags = c->d_status + 1;
    if (cudaMemset(c->d_status, 0, 2 * sizeof(uint32_t)) != cudaSuccess) {
        cudaFree(c->d_status);
        delete c;
        return PC_ERR_CUDA;
    }
    *out = c;
    return PC_OK;
}

void pc_destroy(pc_ctx* c) {
    if (!c) return;
    for (auto& s : c->sources) {
        cudaFree(s.d_off);
        cudaFree(s.d_w);
    }
    for (auto& m : c->dfts) dft_monitor_free(m);
    for (auto& m : c->fluxes) flux_monitor_free(m);
    for (auto& m : c->modes) mode_monitor_free(m);
    cudaFree(c->d_amps);
    cudaFree(c->d_cpml_coef);
    cudaFree(c->d_cpml_slab);
    cudaFree(c->tfsf.d_e1);
    cudaFree(c->tfsf.d_h1);
    cudaFree(c->tfsf.d_inc);
    cudaFree(c->d_status);
    for (cudaEvent_t e : c->prof_ev) cudaEventDestroy(e);
    for (int q = 0; q < 2; ++q)
        if (c->graph[q]) cudaGraphExecDestroy(c->graph[q]);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    cudaFree(c->d_amps_g);
    destroy_fused_state(c);
    destroy_ts_state(c);
    delete c;
}

int pc_set_fields(pc_ctx* c, void* const set0[6], void* const set1[6]) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c || !set0) return PC_ERR_INVALID;
    for (int q = 0; q < 6; ++q) {
        if (!set0[q]) return PC_ERR_INVALID;
        c->F[0][q] = set0[q];
        c->F[1][q] = set1 ? set1[q] : nullptr;
        if (set1 && !set1[q]) return PC_ERR_INVALID;
    }
    if (c->g.sched == PC_SCHED_FUSED && !set1) return PC_ERR_INVALID;
    c->cur = 0;
    c->have_fields = true;
    return PC_OK;
}

int pc_current_set(const pc_ctx* c) { return c ? c->cur : PC_ERR_INVALID; }

int pc_set_current_set(pc_ctx* c, int32_t set) {
    if (!c || set < 0 || set > 1) return PC_ERR_INVALID;
    if (set == 1 && !c->F[1][0]) return PC_ERR_INVALID;
    c->cur = set;
    return PC_OK;
}

int pc_build_coefficients(pc_ctx* c, const double* eps, const double* mu, const double* sig,
                          const double* sigm, double eps0, double mu0, void* const ca[3],
                          void* const cb[3], void* const da[3], void* const db[3], void* stream) {
    if (!c || !(eps0 > 0) || !(mu0 > 0)) return PC_ERR_INVALID;
    return launch_build_coefficients(c->g, eps, mu, sig, sigm, eps0, mu0, ca, cb, da, db,
                                     (cudaStream_t)stream, &c->launches);
}

int pc_set_coefficients(pc_ctx* c, const void* const ca[3], const void* const cb[3],
                        const void* const da[3], const void* const db[3], double da_s, double db_s) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c || !cb) return PC_ERR_INVALID;
    for (int q = 0; q < 3; ++q) {
        if (!cb[q]) return PC_ERR_INVALID;
        c->cb[q] = cb[q];
        c->ca[q] = ca ? ca[q] : nullptr;
        c->da[q] = da ? da[q] : nullptr;
        c->db[q] = db ? db[q] : nullptr;
        if ((c->da[q] == nullptr) != (c->db[q] == nullptr)) return PC_ERR_INVALID;
    }
    c->da_s = da_s;
    c->db_s = db_s;
    c->have_coef = true;
    return PC_OK;
}

size_t pc_cpml_psi_elems(const pc_grid_desc* d, int32_t t) {
    if (validate(d) || t <= 0) return 0;
    return (size_t)psi_layout(*d, t).total;
}

int pc_set_cpml(pc_ctx* c, int32_t t, const double* const b[3], const double* const a[3],
                const double* const kappa[3], void* psi0, void* psi1) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c) return PC_ERR_INVALID;
    if (t <= 0) {
        c->cpml_t = 0;
        return PC_OK;
    }
    if (t > PC_MAX_CPML) return PC_ERR_INVALID;
    if (c->g.mode == PC_MODE_LEGACY) return PC_ERR_INVALID;  // the reference has no CPML
    const pc_grid_desc& g = c->g;
    const int naxes = g.ndim;
    const int n[3] = {g.nx, g.ny, g.ndim == 3 ? g.nz : 0};
    for (int ax = 0; ax < naxes; ++ax) {
        if (!b || !a || !kappa || !b[ax] || !a[ax] || !kappa[ax]) return PC_ERR_INVALID;
        if (2 * t > n[ax]) return PC_ERR_INVALID;
    }
    if (!psi0) return PC_ERR_INVALID;
    if (g.sched == PC_SCHED_FUSED && !psi1) return PC_ERR_INVALID;
    const int64_t total = 3 * ((int64_t)n[0] + n[1] + n[2]);
    const size_t es = (size_t)g.precision;
    std::vector<unsigned char> host(total * es);
    int64_t off = 0;
    for (int ax = 0; ax < 3; ++ax) {
        for (int w = 0; w < 3; ++w) {
            for (int i = 0; i < n[ax]; ++i) {
                double v = w == 0 ? b[ax][i] : (w == 1 ? a[ax][i] : 1.0 / kappa[ax][i]);
                if (es == 8)
                    ((double*)host.data())[off + i] = v;
                else
                    ((float*)host.data())[off + i] = (float)v;
            }
            off += n[ax];
        }
    }
    // compact copy: entries at slab index s (lower slab s < t, upper n - 2t + s)
    std::vector<unsigned char> slab((size_t)9 * 2 * t * es, 0);
    for (int ax = 0; ax < 3; ++ax) {
        for (int w = 0; w < 3; ++w) {
            for (int sidx = 0; sidx < 2 * t; ++sidx) {
                double v = 1.0;
                if (ax < naxes) {
                    const int i = sidx < t ? sidx : n[ax] - 2 * t + sidx;
                    v = w == 0 ? b[ax][i] : (w == 1 ? a[ax][i] : 1.0 / kappa[ax][i]);
                } else if (w == 1) {
                    v = 0.0;
                }
                const size_t o = ((size_t)ax * 3 + w) * 2 * t + sidx;
                if (es == 8)
                    ((double*)slab.data())[o] = v;
                else
                    ((float*)slab.data())[o] = (float)v;
            }
        }
    }
    cudaFree(c->d_cpml_coef);
    cudaFree(c->d_cpml_slab);
    c->d_cpml_coef = nullptr;
    c->d_cpml_slab = nullptr;
    PC_CUDA_CHECK(cudaMalloc(&c->d_cpml_coef, host.size()));
    PC_CUDA_CHECK(cudaMemcpy(c->d_cpml_coef, host.data(), host.size(), cudaMemcpyHostToDevice));
    PC_CUDA_CHECK(cudaMalloc(&c->d_cpml_slab, slab.size()));
    PC_CUDA_CHECK(cudaMemcpy(c->d_cpml_slab, slab.data(), slab.size(), cudaMemcpyHostToDevice));
    c->cpml_t = t;
    c->psi[0] = psi0;
    c->psi[1] = psi1;
    return PC_OK;
}

int pc_add_source(pc_ctx* c, int32_t comp, const int64_t* offsets, const double* weights, int32_t n) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c || comp < 0 || comp > 5 || n <= 0 || !offsets) return PC_ERR_INVALID;
    if ((int)c->sources.size() >= PC_MAX_SOURCES) return PC_ERR_INVALID;
    const int64_t lim = (int64_t)c->g.nx * c->g.ny * c->g.pitch;
    for (int i = 0; i < n; ++i)
        if (offsets[i] < 0 || offsets[i] >= lim) return PC_ERR_INVALID;
    SourceDesc d{};
    d.comp = comp;
    d.n = n;
    PC_CUDA_CHECK(cudaMalloc(&d.d_off, n * sizeof(int64_t)));
    if (cudaMalloc(&d.d_w, n * sizeof(double)) != cudaSuccess) {
        cudaFree(d.d_off);
        return PC_ERR_CUDA;
    }
    std::vector<double> w(n, 1.0);
    if (weights) memcpy(w.data(), weights, n * sizeof(double));
    if (cudaMemcpy(d.d_off, offsets, n * sizeof(int64_t), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d.d_w, w.data(), n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d.d_off);
        cudaFree(d.d_w);
        return PC_ERR_CUDA;
    }
    d.h_off.assign(offsets, offsets + n);
    d.h_w = w;
    c->sources.push_back(d);
    return (int)c->sources.size() - 1;
}

namespace pc {
namespace {

// Steps n (and n + 1) of a pc_step call: stencil, sources (amplitude rows of
// c->d_amps), DFT sampling.  tamp: host TFSF amplitude of the step (or null).
// Advances by two time steps in one launch of the temporally blocked stepper when
// it applies and `left` allows; returns the number of steps taken (or < 0).
int advance(pc_ctx* c, int n, int left, const double* tamp, cudaStream_t s) {
    int rc;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (c->prof_on) {
        if (c->prof_used + 2 > c->prof_ev.size()) {
            for (int q = 0; q < 2; ++q) {
                cudaEvent_t e;
                PC_CUDA_CHECK(cudaEventCreate(&e));
                c->prof_ev.push_back(e);
            }
        }
        ev0 = c->prof_ev[c->prof_used];
        ev1 = c->prof_ev[c->prof_used + 1];
        c->prof_used += 2;
        PC_CUDA_CHECK(cudaEventRecord(ev0, s));
    }
    int k = 1;
    bool fused_sources = false;
    if (c->g.mode == PC_MODE_LEGACY) {
        rc = launch_legacy_step(c, s);
    } else if (left >= 2 && ts_two_step_ok(c)) {
        k = 2;
        rc = launch_ts_step(c, 2, n, s, &fused_sources);
    } else if (ts_eligible(c)) {
        rc = launch_ts_step(c, 1, n, s, &fused_sources);
    } else if (c->g.sched == PC_SCHED_FUSED && c->ade_n == 0 && !c->tfsf.on) {
        rc = launch_fused_step(c, s);
    } else if (c->g.sched == PC_SCHED_FUSED && c->fused_extras && fused_extras_ok(c) && (tamp || !c->tfsf.on)) {
        // ADE / TFSF on the fused schedule: the TFSF line first (incident values of
        // this step), the fused H + E pass (ADE points get the partial update), then
        // the ADE pole terms on the new set
        plan_fused_dft(c);  // plane DFT samples written by the kernels below
        rc = c->tfsf.on ? launch_tfsf_line(c, *tamp, s) : PC_OK;
        if (!rc) rc = launch_fused_step(c, s, tamp);
        if (!rc && c->ade_n > 0) rc = launch_ade_pass(c, c->cur ^ 1, c->cur, s);
    } else {
        rc = launch_split_step(c, s, tamp);
    }
    if (rc) return rc;
    if (ev1) {
        PC_CUDA_CHECK(cudaEventRecord(ev1, s));
        c->prof_steps += k;
    }
    if (!fused_sources) {
        rc = launch_sources(c, n, s);
        if (rc) return rc;
    }
    if (!c->dfts.empty()) {
        rc = dft_after_step(c, s);
        if (rc) return rc;
    }
    if (!c->fluxes.empty()) {
        rc = flux_after_step(c, s);
        if (rc) return rc;
    }
    if (!c->modes.empty()) {
        rc = mode_after_step(c, s);
        if (rc) return rc;
    }
    return k;
}

// The graph of G steps for the current set (captured on first use).  Sources read
// their amplitude rows from c->d_amps_g, which each replay refills.
int ensure_step_graph(pc_ctx* c, int G, size_t ns) {
    const int q = c->cur;
    if (c->graph[q] && c->graph_gen[q] == c->gen && c->graph_G[q] == G) return PC_OK;
    if (c->graph[q]) {
        cudaGraphExecDestroy(c->graph[q]);
        c->graph[q] = nullptr;
    }
    if (!c->cap_stream) PC_CUDA_CHECK(cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    const size_t need = (size_t)G * ns;
    if (need > c->amps_g_cap) {
        cudaFree(c->d_amps_g);
        c->d_amps_g = nullptr;
        c->amps_g_cap = 0;
        PC_CUDA_CHECK(cudaMalloc(&c->d_amps_g, std::max<size_t>(need, 1) * sizeof(double)));
        c->amps_g_cap = need;
    }
    const int cur0 = c->cur;
    const int64_t launches0 = c->launches;
    double* amps0 = c->d_amps;
    std::vector<int> rows0;
    for (auto& m : c->dfts) rows0.push_back(m.rows);
    c->d_amps = c->d_amps_g;
    cudaGraph_t gr = nullptr;
    PC_CUDA_CHECK(cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
    int rc = PC_OK;
    for (int n = 0; n < G;) {
        const int k = advance(c, n, G - n, nullptr, c->cap_stream);
        if (k < 0) {
            rc = k;
            break;
        }
        n += k;
    }
    const cudaError_t e = cudaStreamEndCapture(c->cap_stream, &gr);
    const int64_t nodes = c->launches - launches0;
    c->d_amps = amps0;
    c->cur = cur0;
    c->launches = launches0;
    for (size_t i = 0; i < c->dfts.size(); ++i) c->dfts[i].rows = rows0[i];
    if (rc || e != cudaSuccess) {
        if (gr) cudaGraphDestroy(gr);
        cudaGetLastError();
        return rc ? rc : PC_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(&c->graph[q], gr, 0);
    cudaGraphDestroy(gr);
    if (ei != cudaSuccess) {
        c->graph[q] = nullptr;
        cudaGetLastError();
        return PC_ERR_CUDA;
    }
    c->graph_gen[q] = c->gen;
    c->graph_G[q] = G;
    c->graph_nodes[q] = nodes;
    return PC_OK;
}

}  // namespace
}  // namespace pc

int pc_step(pc_ctx* c, int32_t nsteps, const double* amps, void* stream) {
    if (!c || nsteps < 0) return PC_ERR_INVALID;
    if (!c->have_fields || !c->have_coef) return PC_ERR_STATE;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t ns = c->sources.size();
    const size_t ncol = ns + (c->tfsf.on ? 1 : 0);  // the TFSF amplitude is the last column
    if (c->tfsf.on && !amps) return PC_ERR_INVALID;
    if (ns > 0) {
        if (!amps) return PC_ERR_INVALID;
        const size_t need = (size_t)nsteps * ns;
        if (ncol != ns) {  // repack the source columns (the kernel reads a [nsteps][ns] table)
            c->amps_host.resize(need);
            for (int n = 0; n < nsteps; ++n)
                for (size_t q = 0; q < ns; ++q) c->amps_host[(size_t)n * ns + q] = amps[(size_t)n * ncol + q];
        }
        const double* src_tab = ncol != ns ? c->amps_host.data() : amps;
        if (need > c->amps_cap) {
            PC_CUDA_CHECK(cudaStreamSynchronize(s));
            cudaFree(c->d_amps);
            c->d_amps = nullptr;
            c->amps_cap = 0;
            PC_CUDA_CHECK(cudaMalloc(&c->d_amps, need * sizeof(double)));
            c->amps_cap = need;
        }
        if (need) PC_CUDA_CHECK(cudaMemcpyAsync(c->d_amps, src_tab, need * sizeof(double), cudaMemcpyHostToDevice, s));
        if (ncol != ns) PC_CUDA_CHECK(cudaStreamSynchronize(s));  // amps_host is reused by the next call
    }
    // the time loop replays a captured graph of G steps where it can: no per-step
    // host data (TFSF amplitudes, profiling events), DFT rings at a batch boundary,
    // and the launch setup done by an earlier eager step of the same configuration
    const int G = c->graph_steps;
    const bool graphable = G > 0 && G % 16 == 0 && !c->prof_on && !c->tfsf.on;
    int n = 0;
    while (n < nsteps) {
        bool rows0 = true;
        for (auto& m : c->dfts) rows0 = rows0 && m.rows == 0;
        if (graphable && c->warm_gen == c->gen && rows0 && nsteps - n >= G) {
            const int rc = ensure_step_graph(c, G, ns);
            if (rc == PC_OK) {
                if (ns)
                    PC_CUDA_CHECK(cudaMemcpyAsync(c->d_amps_g, c->d_amps + (size_t)n * ns, (size_t)G * ns * sizeof(double),
                                                  cudaMemcpyDeviceToDevice, s));
                PC_CUDA_CHECK(cudaGraphLaunch(c->graph[c->cur], s));
                c->launches += c->graph_nodes[c->cur];
                n += G;
                continue;
            }
            c->graph_steps = 0;  // capture is not possible here: stay eager
        }
        const double* tamp = c->tfsf.on ? &amps[(size_t)n * ncol + ns] : nullptr;
        // eager steps: the first one of a configuration runs alone (first-launch
        // setup) so that a captured graph never holds it
        const int k = advance(c, n, c->warm_gen == c->gen ? nsteps - n : std::min(nsteps - n, 2), tamp, s);
        if (k < 0) return k;
        c->warm_gen = c->gen;
        n += k;
    }
    return PC_OK;
}

int pc_add_dft(pc_ctx* c, int32_t comp, const int64_t* offsets, int32_t npts, const double* omega, int32_t nf,
               double dt, double t0, void* d_acc) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c || comp < 0 || comp > 5) return PC_ERR_INVALID;
    DftMonitor m{};
    const int rc = dft_monitor_init(m, comp, offsets, npts, omega, nf, dt, t0, d_acc,
                                    (int64_t)c->g.nx * c->g.ny * c->g.pitch);
    if (rc) return rc;
    m.plane_k = -1;
    if (c->g.ndim == 3 && comp < 3 && offsets[0] >= 0 && offsets[0] < c->g.nz) {
        // a whole z-plane in (i, j) order?
        const int64_t P = c->g.pitch, k = offsets[0];
        int ny = 1;
        while (ny < npts && offsets[ny] == offsets[ny - 1] + P) ++ny;
        const int nx = npts / ny;
        bool plane = ny <= c->g.ny && nx <= c->g.nx && (int64_t)nx * ny == npts;
        for (int i = 0; plane && i < nx; ++i)
            for (int j = 0; plane && j < ny; ++j)
                plane = offsets[(int64_t)i * ny + j] == ((int64_t)i * c->g.ny + j) * P + k;
        if (plane) {
            m.plane_k = (int)k;
            m.plane_nx = nx;
            m.plane_ny = ny;
        }
    }
    c->dfts.push_back(m);
    return (int)c->dfts.size() - 1;
}

int pc_set_ade(pc_ctx* c, int32_t n, const pc_ade_region* regs, double eps0) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c || n < 0 || n > PC_MAX_ADE_REGIONS || (n > 0 && !regs) || !(eps0 > 0)) return PC_ERR_INVALID;
    if (n > 0 && c->g.mode == PC_MODE_LEGACY) return PC_ERR_INVALID;  // no ADE coupling in the reference
    const double dt = c->g.dt;
    for (int r = 0; r < n; ++r) {
        const pc_ade_region& R = regs[r];
        if (R.npoles < 0 || R.npoles > PC_MAX_ADE_POLES) return PC_ERR_INVALID;
        for (int a = 0; a < 3; ++a)
            if (R.box[2 * a] < 0 || R.box[2 * a + 1] < R.box[2 * a]) return PC_ERR_INVALID;
        // E+ = (ce E + S - sum aux) / den   (see the oracle's ade_e_coefficients)
        double den = R.eps_inf, ce = R.eps_inf;
        for (int p = 0; p < R.npoles; ++p) {
            if (R.kind[p] == 0) {
                den += R.c0[p];
                ce -= R.c1[p];
            } else if (R.kind[p] == 1) {
                den += dt * R.c0[p] / 4.0;
                ce -= dt * R.c0[p] / 4.0;
            } else if (R.kind[p] == 2) {
                den += R.c0[p] / 2.0;
                ce -= R.c0[p] / 2.0;
            } else {
                return PC_ERR_INVALID;
            }
            for (int comp = 0; comp < 3; ++comp) {
                if (!R.aux[comp][p][0]) return PC_ERR_INVALID;
                if (R.kind[p] == 0 && !R.aux[comp][p][1]) return PC_ERR_INVALID;
            }
        }
        c->ade[r] = R;
        c->ade_ce[r] = ce / den;
        c->ade_inv[r] = 1.0 / den;
    }
    c->ade_n = n;
    c->ade_sdt = dt / eps0;
    return PC_OK;
}

int pc_set_tfsf(pc_ctx* c, int32_t k0, int32_t direction, int32_t polarization, int32_t m0, int32_t aux_len,
                double eps_b, double eps0) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c || c->g.ndim != 3 || c->g.mode != PC_MODE_CORRECTED) return PC_ERR_INVALID;
    if (direction != 1 && direction != -1) return PC_ERR_INVALID;
    if (polarization != 0 && polarization != 1) return PC_ERR_INVALID;
    if (k0 < 1 || k0 > c->g.nz - 3 || m0 < 1 || aux_len < m0 + 3 || !(eps_b > 0) || !(eps0 > 0))
        return PC_ERR_INVALID;
    const size_t es = (size_t)c->g.precision;
    cudaFree(c->tfsf.d_e1);
    cudaFree(c->tfsf.d_h1);
    cudaFree(c->tfsf.d_inc);
    c->tfsf = TfsfState{};
    PC_CUDA_CHECK(cudaMalloc(&c->tfsf.d_e1, aux_len * es));
    PC_CUDA_CHECK(cudaMalloc(&c->tfsf.d_h1, aux_len * es));
    PC_CUDA_CHECK(cudaMalloc(&c->tfsf.d_inc, 2 * es));
    PC_CUDA_CHECK(cudaMemset(c->tfsf.d_e1, 0, aux_len * es));
    PC_CUDA_CHECK(cudaMemset(c->tfsf.d_h1, 0, aux_len * es));
    PC_CUDA_CHECK(cudaMemset(c->tfsf.d_inc, 0, 2 * es));
    c->tfsf.on = true;
    c->tfsf.k0 = k0;
    c->tfsf.dir = direction;
    c->tfsf.pol = polarization;
    c->tfsf.m0 = m0;
    c->tfsf.M = aux_len;
    c->tfsf.cb1 = c->g.dt / (eps0 * eps_b);
    return PC_OK;
}

int pc_dft_flush(pc_ctx* c, int32_t id, void* stream) {
    if (!c || id < 0 || id >= (int)c->dfts.size()) return PC_ERR_INVALID;
    return dft_flush_monitor(c, c->dfts[id], (cudaStream_t)stream);
}

int pc_status(pc_ctx* c, uint32_t* flags, void* stream) {
    if (!c || !flags) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    PC_CUDA_CHECK(cudaMemcpyAsync(flags, c->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PC_CUDA_CHECK(cudaMemsetAsync(c->d_status, 0, sizeof(uint32_t), s));
    PC_CUDA_CHECK(cudaStreamSynchronize(s));
    return PC_OK;
}

int64_t pc_launch_count(const pc_ctx* c) { return c ? c->launches : -1; }

int pc_set_tuning(pc_ctx* c, int32_t key, int64_t value) {
    if (c) ++c->gen;  // captured time loops are stale
    if (!c) return PC_ERR_INVALID;
    switch (key) {
        case PC_TUNE_FUSED_CHUNK:
            if (value < 0 || value > c->g.nx) return PC_ERR_INVALID;
            c->fused_cx = (int)value;
            return PC_OK;
        case PC_TUNE_FUSED_CHUNK_EDGE:
            if (value < 0 || value > c->g.nx) return PC_ERR_INVALID;
            c->fused_cx_edge = (int)value;
            return PC_OK;
        case PC_TUNE_FUSED_SPLIT:
            if (value < 0 || value > 2) return PC_ERR_INVALID;
            c->fused_split = (int)value;
            return PC_OK;
        case PC_TUNE_FUSED_UNIFIED:
            if (value < 0 || value > 1) return PC_ERR_INVALID;
            c->fused_unified = (int)value;
            return PC_OK;
        case PC_TUNE_GRAPH_STEPS:
            if (value < 0 || value % 16 != 0 || value > (1 << 20)) return PC_ERR_INVALID;
            c->graph_steps = (int)value;
            return PC_OK;
        case PC_TUNE_TS_STEPS:
            if (value < 0 || value > 2) return PC_ERR_INVALID;
            c->ts_k = (int)value;
            return PC_OK;
        case PC_TUNE_TS_CHUNK:
            if (value < 0 || value > c->g.nx) return PC_ERR_INVALID;
            c->ts_cx = (int)value;
            return PC_OK;
        case PC_TUNE_TS_ORDER:
            if (value < 0 || value > 2) return PC_ERR_INVALID;
            c->ts_order = (int)value;
            return PC_OK;
        case PC_TUNE_FUSED_EXTRAS:
            if (value < 0 || value > 1) return PC_ERR_INVALID;
            c->fused_extras = (int)value;
            return PC_OK;
        default:
            return PC_ERR_INVALID;
    }
}

int64_t pc_get_tuning(const pc_ctx* c, int32_t key) {
    if (!c) return PC_ERR_INVALID;
    if (key == PC_TUNE_FUSED_CHUNK) return c->fused_cx;
    if (key == PC_TUNE_FUSED_CHUNK_EDGE) return c->fused_cx_edge;
    if (key == PC_TUNE_FUSED_SPLIT) return c->fused_split;
    if (key == PC_TUNE_FUSED_UNIFIED) return c->fused_unified;
    if (key == PC_TUNE_GRAPH_STEPS) return c->graph_steps;
    if (key == PC_TUNE_TS_STEPS) return c->ts_k;
    if (key == PC_TUNE_TS_CHUNK) return c->ts_cx;
    if (key == PC_TUNE_TS_ORDER) return c->ts_order;
    if (key == PC_TUNE_TS_ACTIVE) return ts_eligible(c) ? 1 : 0;
    if (key == PC_TUNE_FUSED_EXTRAS) return c->fused_extras;
    return PC_ERR_INVALID;
}

int pc_profile(pc_ctx* c, int32_t enable) {
    if (!c) return PC_ERR_INVALID;
    c->prof_on = enable != 0;
    c->prof_used = 0;
    c->prof_steps = 0;
    return PC_OK;
}

int pc_profile_read(pc_ctx* c, double* total_ms, int64_t* count) {
    if (!c || !total_ms || !count) return PC_ERR_INVALID;
    double tot = 0.0;
    for (size_t q = 0; q + 1 < c->prof_used; q += 2) {
        PC_CUDA_CHECK(cudaEventSynchronize(c->prof_ev[q + 1]));
        float ms = 0.f;
        PC_CUDA_CHECK(cudaEventElapsedTime(&ms, c->prof_ev[q], c->prof_ev[q + 1]));
        tot += ms;
    }
    *total_ms = tot;
    *count = (int64_t)(c->prof_used / 2);
    c->prof_used = 0;
    c->prof_steps = 0;
    return PC_OK;
}

int64_t pc_profile_steps(const pc_ctx* c) { return c ? c->prof_steps : PC_ERR_INVALID; }

}  // extern "C"
