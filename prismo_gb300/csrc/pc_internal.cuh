// Internal declarations shared by the libprismo_cuda translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/prismo_cuda.h"

#define PC_MAX_SOURCES 64
#define PC_MAX_CPML 64  // maximum CPML thickness in cells

namespace pc {

// Psi slot numbering inside each axis block (four components per axis).
//   x: Eyx Ezx Hyx Hzx   y: Exy Ezy Hxy Hzy   z: Exz Eyz Hxz Hyz
enum { SX_EY = 0, SX_EZ = 1, SX_HY = 2, SX_HZ = 3 };
enum { SY_EX = 0, SY_EZ = 1, SY_HX = 2, SY_HZ = 3 };
enum { SZ_EX = 0, SZ_EY = 1, SZ_HX = 2, SZ_HY = 3 };

struct SourceDesc {
    int comp;
    int n;
    int64_t* d_off;   // device offsets
    double* d_w;      // device weights (float64, converted in-kernel)
    std::vector<int64_t> h_off;  // host copies (the fused-source table of stepper_ts.cu)
    std::vector<double> h_w;
};

// One DFT monitor: samples of `comp` at `npts` element offsets, accumulated for
// `nf` frequencies (see dft.cu).
struct DftMonitor {
    int comp, npts, nf, T, rows;
    double dt;
    int64_t* d_off;   // [npts] element offsets (ctx-owned)
    float* d_ring;    // [T][npts] samples of the pending batch (ctx-owned)
    float2* d_table;  // [T][nf] float32 phases of the batch (ctx-owned)
    double2* d_state; // [nf] float64 phase of the next sample (ctx-owned)
    double2* d_rot;   // [nf] exp(-i w dt) (ctx-owned)
    float4* d_acc;    // [nf][npts] (sum re, sum im, comp re, comp im), caller-owned
    // a whole z-plane of an E component: point i * plane_ny + j is cell (i, j, plane_k)
    // for i < plane_nx, j < plane_ny (plane_k = -1: any other point set)
    int plane_k, plane_nx, plane_ny;
    bool fused;       // sampled by the stepping kernels this step (no dft_sample launch)
    int fused_where;  // 1: by the fused H + E kernel, 2: by the ADE pole pass
};

// Plane DFT monitors whose samples a stepping kernel writes into the ring row of
// the current step (see plan_fused_dft).
#define PC_MAX_FUSED_DFT 2
template <typename T>
struct KernelDft {
    int n;
    int comp[PC_MAX_FUSED_DFT], k[PC_MAX_FUSED_DFT], nx[PC_MAX_FUSED_DFT], ny[PC_MAX_FUSED_DFT];
    float* row[PC_MAX_FUSED_DFT];
};

// Flux plane: per step, sum over its points of (F0 F1 - F2 F3) times `scale`
// (the normal Poynting component of the tangential fields times the cell area)
// appended to a float64 history at a device counter.
struct FluxMonitor {
    int comp[4], npts;
    double scale;
    int64_t* d_off;     // [4][npts] element offsets (ctx-owned)
    int64_t* d_count;   // steps sampled so far (ctx-owned)
    double* d_hist;     // [capacity], caller-owned
    int64_t capacity;
};

// Mode-expansion plane: per step and mode m, a_m = sum over c, p of w[m][c][p]
// F_c(p) (complex weights from the mode profile) appended to a complex history
// [capacity][nmodes] at a device counter.
struct ModeMonitor {
    int comp[4], npts, nmodes;
    int64_t* d_off;     // [4][npts] (ctx-owned)
    double2* d_w;       // [nmodes][4][npts] (ctx-owned)
    int64_t* d_count;   // (ctx-owned)
    double2* d_hist;    // [capacity][nmodes], caller-owned
    int64_t capacity;
    double* d_omega;    // spectrum scratch (ctx-owned)
    int omega_cap;
};

#define PC_MAX_ADE_REGIONS 2
#define PC_MAX_ADE_POLES 4

// Device view of the dispersive regions (see pc_ade_region in the header).
template <typename T>
struct AdeArgs {
    int nreg;
    int box[PC_MAX_ADE_REGIONS][6];
    int npoles[PC_MAX_ADE_REGIONS];
    int kind[PC_MAX_ADE_REGIONS][PC_MAX_ADE_POLES];
    T ce[PC_MAX_ADE_REGIONS];   // coefficient of E^n
    T inv[PC_MAX_ADE_REGIONS];  // 1 / denominator
    T sdt;                       // dt / eps0 (curl -> S)
    T dt;
    T c0[PC_MAX_ADE_REGIONS][PC_MAX_ADE_POLES], c1[PC_MAX_ADE_REGIONS][PC_MAX_ADE_POLES];
    T c2[PC_MAX_ADE_REGIONS][PC_MAX_ADE_POLES], c3[PC_MAX_ADE_REGIONS][PC_MAX_ADE_POLES];
    T* aux[PC_MAX_ADE_REGIONS][3][PC_MAX_ADE_POLES][2];
};

// TFSF plane source state (see tfsf.cu).
struct TfsfState {
    bool on;
    int k0, dir, pol, m0, M;
    double cb1;
    void* d_e1;  // auxiliary E line [M] (ctx-owned)
    void* d_h1;  // auxiliary H line [M] (ctx-owned)
    void* d_inc; // [2]: incident E at step n and incident H at n+1/2 at the plane
                 // (written by tfsf_line for the fused schedule; ctx-owned)
};

// Geometry of the slab-only psi storage.  Axis a keeps four slots; the lower
// slab index s = idx (idx < t), the upper s = idx - (n - 2t) (idx >= n - t).
struct PsiLayout {
    int t;
    int64_t slot_elems[3];  // elements per slot for axis x, y, z
    int64_t axis_base[3];   // element offset of each axis block
    int64_t total;
};

PsiLayout psi_layout(const pc_grid_desc& g, int t);

template <typename T>
struct CpmlArgs {
    int t;
    const T* b[3];     // recursion decay, length n_axis
    const T* a[3];     // recursion gain, length n_axis
    const T* kinv[3];  // 1/kappa, length n_axis
    const T* slabc;    // compact slab coefficients [axis][b, a, kinv][2t]
    const T* psi_in;   // read set
    T* psi_out;        // write set (== psi_in for in-place schedules)
    int64_t slot_elems[3];
    int64_t axis_base[3];
    int64_t total;     // elements of one psi set (bounds check)
    uint32_t* status;  // PC_STATUS_BOUNDS is set instead of an out-of-range access
};

template <typename T>
struct FieldArgs {
    int nx, ny, nz, pitch;
    T dx, dy, dz;            // spacings (legacy kernels divide, as numpy does)
    T inv_dx, inv_dy, inv_dz;
    const T* Ein[3];
    const T* Hin[3];
    T* Eout[3];
    T* Hout[3];
    const T* ca[3];  // nullable: Ca == 1
    const T* cb[3];
    const T* da[3];  // nullable: scalar da_s
    const T* db[3];  // nullable: scalar db_s
    T da_s, db_s;
    uint32_t* status;
};

}  // namespace pc

struct pc_ctx {
    pc_grid_desc g;
    void* F[2][6];
    int cur;
    bool have_fields;
    bool have_coef;
    const void* ca[3];
    const void* cb[3];
    const void* da[3];
    const void* db[3];
    double da_s, db_s;
    // CPML
    int cpml_t;
    void* psi[2];
    void* d_cpml_coef;  // [3 axes][b, a, kinv][n_axis] in context precision
    void* d_cpml_slab;  // [3 axes][b, a, kinv][2t]: the same values at slab indices only
    // TFSF plane source; its amplitude is the last column of the pc_step table
    pc::TfsfState tfsf;
    // dispersive regions (host copy, converted per launch)
    int ade_n;
    pc_ade_region ade[PC_MAX_ADE_REGIONS];
    double ade_ce[PC_MAX_ADE_REGIONS], ade_inv[PC_MAX_ADE_REGIONS], ade_sdt;
    // sources and DFT monitors
    std::vector<pc::SourceDesc> sources;
    std::vector<pc::DftMonitor> dfts;
    std::vector<pc::FluxMonitor> fluxes;
    std::vector<pc::ModeMonitor> modes;
    double* d_amps;
    size_t amps_cap;
    std::vector<double> amps_host;  // repacked source columns when a TFSF column is present
    // fused schedule: cached tensor maps and the chosen x-chunk length
    void* fused_state;
    int fused_cx;
    int fused_cx_edge;  // x-chunk of tiles that touch a y or z slab (0: fused_cx)
    int fused_split;    // CPML item classes: 0 general only, 1 + single-axis, 2 + two-axis (default)
    int fused_unified;  // every class in one launch (1, default) or one launch per class (0)
    int fused_extras;   // ADE regions and TFSF planes on the fused schedule (1, default) or split (0)
    // temporally blocked stepper (stepper_ts.cu): time steps per launch (0 = off), x-chunk
    void* ts_state;
    int ts_k;
    int ts_cx;
    int ts_order;  // work-item order (see PC_TUNE_TS_ORDER)
    // optional CUDA-event timing of the main stencil launch of every step
    bool prof_on;
    std::vector<cudaEvent_t> prof_ev;  // start/stop pairs, recycled
    size_t prof_used;
    int64_t prof_steps;  // time steps covered by the timed launches since the last read
    // status
    uint32_t* d_status;
    uint32_t* d_legacy_flags;
    int64_t launches;
    // captured time loop (pc_step): graphs of graph_steps steps, one per starting set,
    // valid while `gen` (bumped by every call that changes what a step launches) holds
    int64_t gen;
    int64_t warm_gen;  // gen of the last eager step: first-launch setup has run
    int graph_steps;
    cudaStream_t cap_stream;
    cudaGraphExec_t graph[2];
    int64_t graph_gen[2];
    int graph_G[2];
    int64_t graph_nodes[2];
    double* d_amps_g;  // amplitude rows of the chunk a graph replay runs
    size_t amps_g_cap;
};

// ---- launchers (host functions, defined in the .cu files) -------------------
namespace pc {

int launch_build_coefficients(const pc_grid_desc& g, const double* eps, const double* mu,
                              const double* sig, const double* sigm, double eps0, double mu0,
                              void* const ca[3], void* const cb[3], void* const da[3],
                              void* const db[3], cudaStream_t s, int64_t* launches);

int launch_legacy_step(pc_ctx* c, cudaStream_t s);
int launch_split_step(pc_ctx* c, cudaStream_t s, const double* tfsf_amp = nullptr);
int launch_tfsf_h(pc_ctx* c, cudaStream_t s);
int launch_tfsf_e(pc_ctx* c, double amp, cudaStream_t s);
int launch_sources(pc_ctx* c, int step_in_batch, cudaStream_t s);
int launch_fused_step(pc_ctx* c, cudaStream_t s, const double* tfsf_amp = nullptr);
// The fused schedule with ADE regions and / or a TFSF plane: the stepper needs a
// TFSF plane (if any) clear of the ADE boxes' k ranges.
bool fused_extras_ok(const pc_ctx* c);
// Marks the plane DFT monitors that the fused kernel (planes outside the ADE
// boxes) or the ADE pole pass (planes inside the single ADE box) sample this step;
// only without soft sources, which are added after those kernels.
void plan_fused_dft(pc_ctx* c);
template <typename T>
KernelDft<T> kernel_dft(const pc_ctx* c, int where);
int launch_tfsf_line(pc_ctx* c, double amp, cudaStream_t s);
int launch_ade_pass(pc_ctx* c, int in_set, int out_set, cudaStream_t s);
void destroy_fused_state(pc_ctx* c);
int make_map(CUtensorMap* m, const void* base, const pc_grid_desc& g, int bw, int bh);
bool ts_eligible(const pc_ctx* c);
bool ts_two_step_ok(pc_ctx* c);
int launch_ts_step(pc_ctx* c, int k, int row, cudaStream_t s, bool* fused_sources);
void destroy_ts_state(pc_ctx* c);
int dft_after_step(pc_ctx* c, cudaStream_t s);  // skips the monitors marked fused
int launch_dft_sample_f32(const float* field, DftMonitor& m, int row, cudaStream_t s);
int launch_dft_flush_rows(DftMonitor& m, int rows, cudaStream_t s);
int dft_monitor_init(DftMonitor& m, int comp, const int64_t* offsets, int npts, const double* omega, int nf, double dt,
                     double t0, void* d_acc, int64_t limit);
void dft_monitor_free(DftMonitor& m);
int dft_flush_monitor(pc_ctx* c, DftMonitor& m, cudaStream_t s);
int flux_after_step(pc_ctx* c, cudaStream_t s);
void flux_monitor_free(FluxMonitor& m);
int mode_after_step(pc_ctx* c, cudaStream_t s);
void mode_monitor_free(ModeMonitor& m);

}  // namespace pc

#define PC_CUDA_CHECK(x)                          \
    do {                                          \
        cudaError_t err__ = (x);                  \
        if (err__ != cudaSuccess) return PC_ERR_CUDA; \
    } while (0)
