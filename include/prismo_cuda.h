/*
 * prismo_cuda.h -- C ABI of libprismo_cuda.so, the sm_103a FDTD engine behind
 * Prismo's backend interface.
 *
 * The reference drives its time stepper from Python: `prismo.set_backend()`
 * selects an array provider (backends/backend_manager.py:139-186) and
 * `MaxwellUpdater.step` (core/solver.py:535-552) advances the Yee fields with
 * array slicing.  A "cuda" backend binds these entry points through ctypes from
 * Python; every pointer argument named `d_*` is a device pointer owned by the
 * caller, every other pointer is host memory.
 *
 * Conventions
 *   - Every call returns 0 (PC_OK) or a negative PC_ERR_* code, except
 *     pc_fused_steps_noalloc, which returns the index (0 or 1) of the field set
 *     holding its result, or a negative PC_ERR_* code.
 *   - Field buffers use one padded layout for all six components:
 *       3D: element (i, j, k) at ((i*ny + j) * pitch + k)
 *       2D: element (i, j)    at (i * pitch + j)
 *     with pitch >= the fast extent (nz in 3D, ny in 2D) and a multiple of 32.
 *     Entries outside a component's own shape (core/grid.py:157-168) are zero
 *     and stay zero.
 *   - Component order is Ex, Ey, Ez, Hx, Hy, Hz (index 0..5).
 *   - A context is not thread safe; separate contexts may run on separate
 *     streams.  Device-side problems set bits in a status word (pc_status).
 */
#ifndef PRISMO_CUDA_H
#define PRISMO_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PC_OK 0
#define PC_ERR_INVALID (-1)      /* bad argument / unsupported combination */
#define PC_ERR_CUDA (-2)         /* a CUDA runtime call failed */
#define PC_ERR_TIMEOUT (-3)      /* a bounded device wait ran out */
#define PC_ERR_NONFINITE (-4)    /* NaN/Inf detected in the fields */
#define PC_ERR_STATE (-5)        /* call out of order (e.g. step before set_fields) */

#define PC_STATUS_NONFINITE 0x1u
#define PC_STATUS_TIMEOUT 0x2u
#define PC_STATUS_BOUNDS 0x4u

/* Stepper kinds */
#define PC_MODE_CORRECTED 0 /* stable Yee scheme: H written to [...,1:-1,...] */
#define PC_MODE_LEGACY 1    /* exact core/solver.py:167-456 semantics */

/* Kernel schedule for the corrected 3D stepper */
#define PC_SCHED_AUTO 0
#define PC_SCHED_SPLIT 1 /* separate H and E passes, in place */
#define PC_SCHED_FUSED 2 /* one fused H+E pass per step, ping-pong buffers */

typedef struct pc_grid_desc {
    int32_t ndim;      /* 2 or 3 */
    int32_t nx, ny, nz; /* total Yee dimensions, core/grid.py:122-125 (nz = 1 in 2D) */
    int32_t pitch;     /* elements per fast row of every field buffer */
    int32_t precision; /* 4 = float32, 8 = float64 */
    int32_t mode;      /* PC_MODE_* */
    int32_t sched;     /* PC_SCHED_* */
    double dt, dx, dy, dz;
} pc_grid_desc;

typedef struct pc_ctx pc_ctx;

/* Library version (major*10000 + minor*100 + patch). */
int pc_version(void);

/* Create / destroy a stepping context (replaces the state that
 * MaxwellUpdater.__init__ builds, core/solver.py:42-79). */
int pc_create(const pc_grid_desc* desc, pc_ctx** out);
void pc_destroy(pc_ctx* ctx);

/* Attach field storage: set0/set1 hold device pointers to the six components
 * (Ex..Hz).  set1 may be NULL when the schedule does not ping-pong; the fused
 * schedule writes step n+1 into the other set.  Replaces core/fields.py:64-70. */
int pc_set_fields(pc_ctx* ctx, void* const set0[6], void* const set1[6]);

/* Which set (0 or 1) currently holds the latest fields. */
int pc_current_set(const pc_ctx* ctx);

/* Declare which attached set holds the latest fields (e.g. after rebinding
 * storage whose newest data sits in set 1). */
int pc_set_current_set(pc_ctx* ctx, int32_t set);

/* Build the interpolated update coefficients on the device from cell-centred
 * material arrays (core/solver.py:113-133 and 458-533).  Inputs are float64
 * device arrays of shape (nx, ny, nz), contiguous; any may be NULL (vacuum:
 * eps_rel = mu_rel = 1, sigma = 0).  Outputs use the padded field layout in
 * the context precision; d_ca / d_da / d_db outputs may be NULL to skip. */
int pc_build_coefficients(pc_ctx* ctx, const double* d_eps_rel, const double* d_mu_rel,
                          const double* d_sigma_e, const double* d_sigma_m, double eps0,
                          double mu0, void* const d_ca[3], void* const d_cb[3],
                          void* const d_da[3], void* const d_db[3], void* stream);

/* Attach coefficients for E (Ca may be NULL: treated as 1) and H (arrays may be
 * NULL: the scalars da, db are used for every H point). */
int pc_set_coefficients(pc_ctx* ctx, const void* const d_ca[3], const void* const d_cb[3],
                        const void* const d_da[3], const void* const d_db[3], double da,
                        double db);

/* Number of elements of one psi set for CPML thickness t (both slabs of all
 * three axes, four components per axis). */
size_t pc_cpml_psi_elems(const pc_grid_desc* desc, int32_t thickness);

/* Enable the CPML: per-axis host arrays b, a, kappa of length nx, ny, nz
 * (boundaries/pml.py:117-257 profiles; pass the z arrays as NULL in 2D), and
 * one or two zeroed device psi sets of pc_cpml_psi_elems() elements. */
int pc_set_cpml(pc_ctx* ctx, int32_t thickness, const double* const b[3], const double* const a[3],
                const double* const kappa[3], void* d_psi0, void* d_psi1);

/* Soft source: field[comp][offset[n]] += weight[n] * amplitude(t_{n+1}) after the
 * E update of every step (sources/point.py:47-73, plane_wave.py:184-221).
 * Offsets are element offsets in the padded layout.  Returns the source id
 * (>= 0) or an error. */
int pc_add_source(pc_ctx* ctx, int32_t comp, const int64_t* offsets, const double* weights,
                  int32_t n);

/* Advance nsteps leap-frog steps (H then E then sources), i.e. nsteps calls of
 * MaxwellUpdater.step followed by Source.update_fields (core/simulation.py:147-164).
 * amps: host array [nsteps][nsources] of source amplitudes (may be NULL when
 * there are no sources). */
int pc_step(pc_ctx* ctx, int32_t nsteps, const double* amps, void* stream);

/* Dispersive (ADE) region: E components whose own index lies in
 * [box0,box1) x [box2,box3) x [box4,box5) use the auxiliary-differential-equation
 * update instead of Ca/Cb (materials/ade.py:100-160 recursions with the
 * coefficients of materials/dispersion.py:189-336, coupled to E through the
 * polarisation current):
 *   Lorentz (kind 0): P+ = C0 E+ + C1 E + C2 P + C3 P-       (aux: P, D = P - P-)
 *   Drude   (kind 1): J+ = C1 J + C0 (E+ + E)/2               (aux: J)
 *   Debye   (kind 2): P+ = C1 P + C0 (E+ + E)/2               (aux: P)
 * with eps_inf (E+ - E) + sum dP (or dt J terms) = (dt/eps0) curl H, solved for E+.
 * The Lorentz recursion is carried as P and its last increment D: the same
 * algebra, D+ = C0 E+ + C1 E + (C2 + C3 - 1) P - C3 D and P+ = P + D+, without
 * the float32 cancellation of C2 P + C3 P- (C2 is close to 2 and C3 to -1).
 * aux[c][p][0..1]: caller-owned zeroed device arrays over the box (C order,
 * float context precision), per E component c and pole p. */
typedef struct pc_ade_region {
    int32_t box[6];
    int32_t npoles;
    int32_t kind[4];
    double eps_inf;
    double c0[4], c1[4], c2[4], c3[4];
    void* aux[3][4][2];
} pc_ade_region;

int pc_set_ade(pc_ctx* ctx, int32_t nregions, const pc_ade_region* regions, double eps0);

/* Plane-wave TFSF source on the plane k = k0 (3D, corrected stepper), fed by a
 * 1D auxiliary Yee line of aux_len points with the same dz and dt in a medium of
 * relative permittivity eps_b, sampled at index m0 (replaces the single-plane
 * correction of sources/tfsf.py:258-411).  direction = +1/-1 (propagation along
 * +z/-z), polarization 0 = Ex/Hy, 1 = Ey/Hx.  Its waveform amplitude a(t_{n+1})
 * is the last column of the pc_step amplitude table.  The plane must lie outside
 * the z CPML and dispersive regions. */
int pc_set_tfsf(pc_ctx* ctx, int32_t k0, int32_t direction, int32_t polarization, int32_t m0, int32_t aux_len,
                double eps_b, double eps0);

/* DFT monitor (monitors/field.py:138-143, monitors/dft.py:108-137): after every
 * step (and after the sources) F_f += field(t_{n+1}) exp(-i omega_f t_{n+1}) dt at
 * the npts element offsets of component comp.  t0 is t_{n+1} of the next step.
 * d_acc is caller-owned float [nf][npts][4] = (sum re, sum im, Kahan compensation
 * re, im), zeroed; the estimate is sum - compensation.  Samples are batched (16
 * steps) and folded in with a float64 phase recurrence; call pc_dft_flush before
 * reading d_acc.  Returns the monitor id. */
int pc_add_dft(pc_ctx* ctx, int32_t comp, const int64_t* offsets, int32_t npts, const double* omega,
               int32_t nf, double dt, double t0, void* d_acc);
int pc_dft_flush(pc_ctx* ctx, int32_t id, void* stream);

/* Flux monitor, time domain (monitors/flux.py:110-173 FluxMonitor.update and
 * _compute_power_flow): after every step (after the DFT samples)
 *   d_hist[n] = scale * sum_p (F0 F1 - F2 F3)(p)
 * with F0..F3 the components comps[0..3] at offsets[q * npts + p] (for a plane
 * normal to x: Ey, Hz, Ez, Hy and scale = dy dz), n counting the steps since the
 * monitor was added; steps beyond `capacity` are counted, not stored.  d_hist is
 * caller-owned float64 [capacity].  Returns the monitor id. */
int pc_add_flux(pc_ctx* ctx, const int32_t comps[4], const int64_t* offsets, int32_t npts, double scale,
                double* d_hist, int64_t capacity);
/* Steps sampled so far by flux monitor `id` (synchronises the stream). */
int pc_flux_count(pc_ctx* ctx, int32_t id, int64_t* count, void* stream);
/* Flux monitor, frequency domain (monitors/flux.py:219-285
 * get_frequency_domain_power): flushes the four DFT monitors dft_ids (same points
 * and frequencies, components F0..F3 as above) and writes
 *   d_out[f] = scale / 2 * sum_p Re(F0 F1* - F2 F3*)
 * for every frequency (device float64 [nf]). */
int pc_flux_spectrum(pc_ctx* ctx, const int32_t dft_ids[4], double scale, double* d_out, void* stream);

/* Mode-expansion monitor (monitors/mode_monitor.py:137-199 with
 * utils/mode_matching.py:41-131): after every step, for every mode m
 *   d_hist[n][m] = sum_{q<4, p<npts} w[m][q][p] * F_q(offsets[q * npts + p])
 * (complex weights, float64 (re, im) pairs [nmodes][4][npts]; the host folds the
 * mode profile, the cross-product signs and 1 / (2 P_m) into them), n counting
 * the steps since the monitor was added.  d_hist is caller-owned complex128
 * [capacity][nmodes]; nmodes <= 64.  Returns the monitor id. */
int pc_add_mode_monitor(pc_ctx* ctx, const int32_t comps[4], const int64_t* offsets, int32_t npts, int32_t nmodes,
                        const double* weights, void* d_hist, int64_t capacity);
int pc_mode_count(pc_ctx* ctx, int32_t id, int64_t* count, void* stream);
/* d_out[m][f] = sum_n d_hist[n][m] exp(-i omega_f (t0 + n dt)) dt over the steps
 * sampled so far (mode_monitor.py:171-175; t0 = time of the first sample);
 * omega is a host array; synchronises the stream.  PC_ERR_STATE when more steps
 * were sampled than the history holds. */
int pc_mode_spectrum(pc_ctx* ctx, int32_t id, const double* omega, int32_t nf, double t0, double dt, void* d_out,
                     void* stream);

/* Mode ports (boundaries/mode_port.py:261-429), on device arrays outside a
 * context.  pc_scatter_add: field[off[i]] = field[off[i]] + amp * w[i] computed in
 * float64 and rounded once to the field type (precision 4 or 8); d_off (int64
 * element offsets) and d_w (float64) are device arrays of n entries.
 * pc_plane_overlap: d_out[m] = sum_{q<4, p<npts} w[m][q][p] F_q(off[q*npts + p])
 * for m < nmodes, complex float64 weights [nmodes][4][npts] and output
 * [nmodes] (re, im) on the device. */
int pc_scatter_add(int32_t precision, void* field, const int64_t* d_off, const double* d_w, int64_t n, double amp,
                   void* stream);
int pc_plane_overlap(int32_t precision, const void* const fields[4], const int64_t* d_off, int32_t npts,
                     int32_t nmodes, const void* d_w, void* d_out, void* stream);

/* Anisotropic field update (materials/tensor.py:437-590 AnisotropicUpdater),
 * elementwise over n cells of same-shaped device arrays (precision 4 or 8):
 *   sign +1 (E):  out = F + scale * curl / diag            (diagonal)
 *                 out = F + scale * (M . curl)              (full, M row-major)
 *   sign -1 (H):  out = F - scale * curl / diag, out = F + (-scale) * (M . curl)
 * with scale = dt/eps0 or dt/mu0, the coefficients per cell (device d_coef
 * [3 or 9][n] in the array precision) or uniform (host coef_uniform [3 or 9],
 * used when d_coef is null); M is the inverse tensor.  Rounded in the
 * reference's evaluation order (float64 equals NumPy bit for bit).  out may
 * alias fields. */
int pc_aniso_update(int32_t precision, int32_t diagonal, int32_t sign, const void* const fields[3],
                    const void* const curls[3], void* const out[3], int64_t n, const void* d_coef,
                    const double* coef_uniform, double scale, void* stream);

/* Read and clear the device status word (PC_STATUS_* bits). Synchronises the
 * stream. */
int pc_status(pc_ctx* ctx, uint32_t* flags, void* stream);

/* Number of this library's kernels launched since the context was created. */
int64_t pc_launch_count(const pc_ctx* ctx);

/* Tuning knobs.  PC_TUNE_FUSED_CHUNK: planes along x streamed by one CTA of the
 * fused 3D schedule (0 = automatic choice).  PC_TUNE_FUSED_CHUNK_EDGE: the same
 * for tiles that touch a y or z CPML slab (0 = PC_TUNE_FUSED_CHUNK).
 * PC_TUNE_FUSED_SPLIT: which CPML work items get a kernel variant of their own
 * slab axes (float32 without per-cell H or Ca coefficients): 0 none (one
 * general variant), 1 items on one axis's slabs, 2 also items on two axes' slabs
 * (default).  PC_TUNE_FUSED_UNIFIED: those variants run as one launch that picks
 * the variant per work item (1, default) or as one launch per variant on
 * concurrent streams (0).  PC_TUNE_GRAPH_STEPS: pc_step replays
 * its time loop from a CUDA graph of this many steps (a multiple of 16; 0 = one
 * launch sequence per step), captured on first use after an eager step and
 * re-captured after any call that changes what a step launches.  Steps with a
 * TFSF source or with pc_profile enabled always run eagerly.  Default 64.
 * PC_TUNE_TS_STEPS: time steps per launch of the temporally blocked 3D stepper
 * (float32, lossless non-magnetic media, CPML, soft E sources fused in): 2
 * (default) advances two steps per launch wherever no monitor samples the
 * intermediate step, 1 one step per launch, 0 leaves it off (the fused schedule
 * above runs).  PC_TUNE_TS_CHUNK: its x-chunk length (0 = automatic, 32).
 * PC_TUNE_TS_ORDER: its work-item order: 0 chunk after chunk in grid order, 1
 * the most expensive chunks (those on the x slabs) first and the slower items
 * of a chunk first, 2 (default) every item by its cost.  PC_TUNE_TS_ACTIVE
 * (read only): 1 when the temporally blocked stepper runs for this context's
 * current configuration.  PC_TUNE_FUSED_EXTRAS: 3D grids with ADE regions or a
 * TFSF plane run on the fused schedule (1, default: the TFSF plane corrections
 * and the ADE partial update inside the fused H + E kernel, the ADE pole terms in
 * one pass over each region afterwards; needs the TFSF plane outside the ADE
 * boxes' k ranges; without soft sources, DFT monitors on a whole z-plane of an E
 * component are sampled inside those kernels) or on the split schedule (0). */
#define PC_TUNE_FUSED_CHUNK 1
#define PC_TUNE_GRAPH_STEPS 2
#define PC_TUNE_FUSED_CHUNK_EDGE 3
#define PC_TUNE_FUSED_SPLIT 4
#define PC_TUNE_FUSED_UNIFIED 5
#define PC_TUNE_TS_STEPS 6
#define PC_TUNE_TS_CHUNK 7
#define PC_TUNE_TS_ORDER 8
#define PC_TUNE_TS_ACTIVE 9
#define PC_TUNE_FUSED_EXTRAS 10
int pc_set_tuning(pc_ctx* ctx, int32_t key, int64_t value);
int64_t pc_get_tuning(const pc_ctx* ctx, int32_t key);

/* Time the main stencil launch of every pc_step with a CUDA event pair on the
 * launching stream (enable != 0), and read the summed milliseconds and the
 * number of timed launches since the last read (synchronises the events). */
int pc_profile(pc_ctx* ctx, int32_t enable);
int pc_profile_read(pc_ctx* ctx, double* total_ms, int64_t* count);
/* Time steps covered by the launches timed since the last pc_profile_read (a
 * launch of the temporally blocked stepper covers two); read it before
 * pc_profile_read, which resets it. */
int64_t pc_profile_steps(const pc_ctx* ctx);

/* Allocation-free stepping.  This entry point has no counterpart in the
 * reference; it serves callers that may not allocate device memory: a host
 * application whose device memory is owned entirely by its own pool allocator,
 * or a time loop that must not pay cudaMalloc's latency and device-wide
 * synchronisation.  It runs nsteps of the fused 3D corrected stepper (float32 or
 * float64, vacuum mu, sigma = 0, no CPML and no sources) without a context and
 * without allocating: the caller passes both field sets (set0/set1, six device
 * pointers each, padded layout of this header) and the three Cb arrays; `cur`
 * names the set holding the current fields; the return value is the set that
 * holds the result (>= 0) or a PC_ERR_* code.
 *   - Scratch (the kernel's work-item list and its status word) lives in one
 *     fixed device array of 32768 work items (about 512 KB) that every GPU
 *     loading the library keeps until the process exits.  Grids needing more
 *     work items (more than 32768 tiles of 16 x 32 cells times x-chunks) are
 *     rejected with PC_ERR_INVALID.
 *   - The first call on a device resolves that array's device address (call it
 *     with that device current, and before any stream capture).
 *   - Every call shares the array and resets the status word at its start;
 *     calls that overlap on the GPU race.
 *   - status_out (host, nullable) receives the PC_STATUS_* bits; passing it
 *     synchronises the stream.  Without it, non-finite fields and a bounded
 *     wait that ran out (PC_STATUS_NONFINITE, PC_STATUS_TIMEOUT) are not
 *     reported: the next call clears the word before anyone can read it.
 *   - The device address is cached per device index for the life of the
 *     process; after cudaDeviceReset on a device, do not call this entry point
 *     on that device again. */
int pc_fused_steps_noalloc(const pc_grid_desc* desc, void* const set0[6], void* const set1[6], int32_t cur,
                           const void* const cb[3], int32_t nsteps, void* stream, uint32_t* status_out);

/* ------------------------------------------------------------------------- *
 * Batched 2D sweep.  Replaces the per-design loop of ParameterSweep
 * (optimization/sweep.py:41-195, one Simulation.run per design, sequential or
 * in a process pool) for 2D TE designs (Ez, Hx, Hy; core/solver.py:311-456,
 * corrected stencil) that share dx, dy, dt and the CPML thickness but not their
 * grid size.  All instances advance together: one persistent kernel per pass
 * covers every (instance, tile) item and runs K steps per pass; the time loop
 * is replayed from a captured CUDA graph of G steps.  Float32 fields, lossless
 * non-magnetic media (Ca = 1, Da = 1, Db = db_s).
 *
 * Per-instance device layout (offsets from pc_batch_instance_offsets):
 *   field set: Ez, Hx, Hy, each [nx][pitch] (pitch = ny rounded up to 32),
 *              at field_offset + q * nx * pitch (q = 0, 1, 2)
 *   Cb(Ez):    [nx][pitch] at coef_offset
 * Each instance has one soft Ez line source (Ez index src_x, y in
 * [src_y0, src_y0 + src_n)) with per-point weights, all driven by one amplitude
 * table a(t_{n+1}) (sources/point.py:62-73), and up to four DFT port lines of Ez
 * (x = port_x, y in [port_y0, port_y0 + port_n)) at shared frequencies.
 * ------------------------------------------------------------------------- */
typedef struct pc_batch pc_batch;

typedef struct pc_batch_instance {
    int32_t nx, ny;               /* total Yee dimensions (2D) */
    int32_t src_x, src_y0, src_n; /* soft Ez line source */
    int32_t nport;                /* 0..4 */
    int32_t port_x[4], port_y0[4], port_n[4];
} pc_batch_instance;

typedef struct pc_batch_layout {
    int64_t field_elems;  /* floats in one field set (all instances) */
    int64_t coef_elems;   /* floats in the Cb(Ez) buffer */
    int64_t psi_elems;    /* floats in one CPML auxiliary buffer */
    int64_t weight_elems; /* source weights of all instances (doubles) */
    int64_t dft_points;   /* port points of all instances */
} pc_batch_layout;

/* Describe the batch (host only, plus small descriptor buffers).  db_s =
 * dt / mu0.  `lay` receives the sizes of the caller-owned buffers. */
int pc_batch_create(int32_t ninst, const pc_batch_instance* inst, int32_t cpml_t, double dx, double dy, double dt,
                    double db_s, pc_batch** out, pc_batch_layout* lay);
/* out = {field offset, pitch, coef offset, first weight, first DFT point} */
int pc_batch_instance_offsets(const pc_batch* b, int32_t i, int64_t out[5]);
/* Two zeroed field sets, the Cb buffer and (cpml_t > 0) two zeroed CPML buffers. */
int pc_batch_bind(pc_batch* b, void* d_set0, void* d_set1, void* d_cb, void* d_psi0, void* d_psi1);
/* Cb(Ez) of instance i from its cell-centred relative permittivity d_eps
 * (device float64 [nx][ny]), core/solver.py:113-133 + 4-point Ez average. */
int pc_batch_build_coefficients(pc_batch* b, int32_t i, const double* d_eps, double eps0, void* stream);
/* CPML recursion coefficients by slab index (2 * cpml_t entries each: lower
 * slab cells 0..t-1, then upper slab cells n-t..n-1), shared by both axes. */
int pc_batch_set_cpml(pc_batch* b, const double* bcoef, const double* acoef, const double* kappa);
/* Source weights (weight_elems doubles, instance-major) and the amplitude table
 * a(t_{n+1}) of steps 0..namps-1 (0 after the table). */
int pc_batch_set_sources(pc_batch* b, const double* weights, const double* amps, int32_t namps);
/* Port DFT of every instance's port lines (Ez) at nf angular frequencies; t0 is
 * t_{n+1} of the next step; d_acc is caller-owned zeroed float
 * [nf][dft_points][4] as in pc_add_dft.  Point order: instance, port, y. */
int pc_batch_set_dft(pc_batch* b, const double* omega, int32_t nf, double t0, void* d_acc);
/* Kernel variants: tile (TX x TY cells) and steps per pass K. */
int pc_batch_num_variants(void);
int pc_batch_variant_info(int32_t variant, int32_t out[3]);
/* graph_steps: steps per captured graph (a multiple of 16 with an even number of
 * passes), 0 = no graph. */
int pc_batch_set_tuning(pc_batch* b, int32_t variant, int32_t graph_steps);
int pc_batch_get_tuning(const pc_batch* b, int32_t* variant, int32_t* graph_steps);
/* Time `passes` dry passes (no source, no sampling; the current state is not
 * changed) of every variant and select the fastest per step; ms_per_step
 * (nullable) receives pc_batch_num_variants() values. */
int pc_batch_autotune(pc_batch* b, int32_t passes, float* ms_per_step, void* stream);
int pc_batch_step(pc_batch* b, int32_t nsteps, void* stream);
int pc_batch_dft_flush(pc_batch* b, void* stream);
int pc_batch_current_set(const pc_batch* b);
/* Status words (PC_STATUS_* bits).  pc_batch_status reads the batch's word;
 * pc_batch_instance_status reads one word per instance into flags[ninst] and
 * clears them (synchronises the stream).  A pass that stores a NaN or Inf in
 * an instance's Ez sets PC_STATUS_NONFINITE in that instance's word and in the
 * batch word, so a caller can re-run just the failed designs on the
 * per-simulation path (ParameterSweep marks a failed point and goes on,
 * optimization/sweep.py:183-195). */
int pc_batch_status(pc_batch* b, uint32_t* flags, void* stream);
int pc_batch_instance_status(pc_batch* b, uint32_t* flags, void* stream);
int64_t pc_batch_launch_count(const pc_batch* b);
int64_t pc_batch_steps_done(const pc_batch* b);
void pc_batch_destroy(pc_batch* b);

/* ------------------------------------------------------------------------- *
 * Surrogate network.  No counterpart in the reference (it has no learned
 * model): an ensemble of `members` MLPs dims[0] -> dims[1] -> dims[2] -> dims[3]
 * -> dims[4] with SiLU after the three hidden layers, bf16 weights on the
 * tensor cores with float32 accumulation (forward activations as bf16 hi/lo
 * pairs, backward in bf16), float32 master parameters and Adam.
 * dims[0] <= 32 (padded to 32 internally); dims[1..4]
 * multiples of 32.  Batches: 1..max_batch rows for the forward pass, multiples
 * of 32 for training; max_batch a multiple of 32.
 *
 * Parameter vector of one member (P floats, pc_mlp_param_count): for layer
 * l = 0..3 the weight [n_l][k_l] (row-major, k_0 = 32 with columns >= dims[0]
 * zero) at w_off, then the bias [n_l] at b_off (pc_mlp_param_layout).  Host
 * parameter and gradient arrays are [members][P].  Device inputs x are
 * [members][batch][dims[0]] float32, targets and outputs [members][batch][dims[4]].
 * ------------------------------------------------------------------------- */
typedef struct pc_mlp pc_mlp;

int pc_mlp_create(int32_t members, int32_t max_batch, const int32_t dims[5], pc_mlp** out);
int64_t pc_mlp_param_count(const pc_mlp* n);
/* out = {w_off, b_off, n, k} of layer l */
int pc_mlp_param_layout(const pc_mlp* n, int32_t layer, int64_t out[4]);
/* Load the float32 masters of every member (resets Adam's moments and step). */
int pc_mlp_set_params(pc_mlp* n, const float* host);
int pc_mlp_get_params(const pc_mlp* n, float* host);
int pc_mlp_get_grads(const pc_mlp* n, float* host);
int pc_mlp_forward(pc_mlp* n, const float* d_x, int32_t batch, float* d_y, void* stream);
/* Forward + backward of the mean-squared error mean((y - t)^2) per member;
 * gradients land in the gradient buffer, d_loss (device, nullable) gets
 * [members] losses. */
int pc_mlp_gradients(pc_mlp* n, const float* d_x, const float* d_t, int32_t batch, float* d_loss, void* stream);
/* pc_mlp_gradients followed by one Adam step (bias-corrected). */
int pc_mlp_train_step(pc_mlp* n, const float* d_x, const float* d_t, int32_t batch, float lr, float beta1,
                      float beta2, float eps, float* d_loss, void* stream);
int64_t pc_mlp_launch_count(const pc_mlp* n);
/* Where the products run: the 5th-generation tensor cores (tcgen05.mma with a
 * tensor-memory accumulator; 1: every product whose shape fits), mma.sync (0),
 * or (2, the default) tcgen05 for launches of at least 64 of its 128 x 256 tiles
 * and mma.sync below that.  Output widths that are not multiples of 256, and
 * unaligned outputs, always use mma.sync. */
int pc_mlp_set_tensor_path(pc_mlp* n, int32_t tcgen05);
/* Read the status word (PC_STATUS_TIMEOUT: a bounded wait for the tensor cores
 * ran out).  Synchronises the stream. */
int pc_mlp_status(pc_mlp* n, uint32_t* flags, void* stream);
void pc_mlp_destroy(pc_mlp* n);

#ifdef __cplusplus
}
#endif

#endif /* PRISMO_CUDA_H */
