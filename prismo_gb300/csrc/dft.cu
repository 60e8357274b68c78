// On-the-fly DFT monitors: F_f += f(t_{n+1}) exp(-i w_f t_{n+1}) dt for every
// monitored point, the running sum of monitors/field.py:138-143 (FieldMonitor with
// frequencies=) and monitors/dft.py:108-137.
//
// GB300 design: sampling and accumulation are separated so that the complex
// accumulators (4 floats per point and frequency) are touched once per T steps
// instead of every step.
//   * dft_sample (every step, after the sources): copy the monitored points of the
//     current field set into row (n mod T) of a sample ring [T][npts].
//   * dft_phase (every T steps): extend the float64 phase recurrence
//     ph_f <- ph_f * exp(-i w_f dt) over the T steps of the batch, writing a
//     float32 table [T][nf] and keeping the float64 state for the next batch.
//   * dft_flush: for each (f, point) the batch sum S = sum_t x_t ph_{t,f} is formed
//     in float32 registers, then S*dt is added to the accumulator with Kahan
//     compensation (sum, compensation) in float32.
#include "pc_internal.cuh"

namespace pc {
namespace {

template <typename T>
__global__ void dft_sample(const T* __restrict__ field, const int64_t* __restrict__ off, int npts,
                           float* __restrict__ ring, int row) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npts; i += gridDim.x * blockDim.x)
        ring[(int64_t)row * npts + i] = static_cast<float>(field[off[i]]);
}

// one thread per frequency: float64 recurrence over the rows of the batch
__global__ void dft_phase(double2* __restrict__ state, const double2* __restrict__ rot, int nf, int rows,
                          float2* __restrict__ table) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    double2 p = state[f];
    const double2 r = rot[f];
    for (int t = 0; t < rows; ++t) {
        table[t * nf + f] = make_float2((float)p.x, (float)p.y);
        const double re = p.x * r.x - p.y * r.y;
        const double im = p.x * r.y + p.y * r.x;
        p = make_double2(re, im);
    }
    state[f] = p;
}

// grid: (point blocks, frequency blocks); each thread one (f, point); the batch's
// samples of the point are read once per thread from the ring (L1/L2 resident).
__global__ void dft_flush(const float* __restrict__ ring, int npts, int rows, const float2* __restrict__ table,
                          int nf, float dt, float4* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= npts || f >= nf) return;
    float sr = 0.f, si = 0.f;
    for (int t = 0; t < rows; ++t) {
        const float x = ring[(int64_t)t * npts + i];
        const float2 ph = table[t * nf + f];
        sr = fmaf(x, ph.x, sr);
        si = fmaf(x, ph.y, si);
    }
    float4 a = acc[(int64_t)f * npts + i];  // (sum_re, sum_im, comp_re, comp_im)
    // Kahan: y = v - c; t = s + y; c = (t - s) - y; s = t
    const float yr = sr * dt - a.z;
    const float tr = a.x + yr;
    a.z = (tr - a.x) - yr;
    a.x = tr;
    const float yi = si * dt - a.w;
    const float ti = a.y + yi;
    a.w = (ti - a.y) - yi;
    a.y = ti;
    acc[(int64_t)f * npts + i] = a;
}

}  // namespace

// launch helpers shared with the batched sweep (batch.cu)
int launch_dft_sample_f32(const float* field, DftMonitor& m, int row, cudaStream_t s) {
    const int threads = 256;
    const int blocks = (m.npts + threads - 1) / threads < 1024 ? (m.npts + threads - 1) / threads : 1024;
    dft_sample<float><<<blocks, threads, 0, s>>>(field, m.d_off, m.npts, m.d_ring, row);
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

int launch_dft_flush_rows(DftMonitor& m, int rows, cudaStream_t s) {
    dft_phase<<<(m.nf + 127) / 128, 128, 0, s>>>(m.d_state, m.d_rot, m.nf, rows, m.d_table);
    dim3 grd((m.npts + 255) / 256, m.nf);
    dft_flush<<<grd, 256, 0, s>>>(m.d_ring, m.npts, rows, m.d_table, m.nf, (float)m.dt, m.d_acc);
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

int dft_after_step(pc_ctx* c, cudaStream_t s) {
    for (auto& m : c->dfts) {
        if (m.fused) {  // the stepping kernels wrote ring row m.rows
            m.fused = false;
            if (++m.rows == m.T) {
                const int rc = dft_flush_monitor(c, m, s);
                if (rc) return rc;
            }
            continue;
        }
        const int threads = 256;
        const int blocks = (m.npts + threads - 1) / threads < 1024 ? (m.npts + threads - 1) / threads : 1024;
        if (c->g.precision == 8)
            dft_sample<double><<<blocks, threads, 0, s>>>(static_cast<const double*>(c->F[c->cur][m.comp]), m.d_off,
                                                          m.npts, m.d_ring, m.rows);
        else
            dft_sample<float><<<blocks, threads, 0, s>>>(static_cast<const float*>(c->F[c->cur][m.comp]), m.d_off,
                                                         m.npts, m.d_ring, m.rows);
        ++c->launches;
        if (++m.rows == m.T) {
            int rc = dft_flush_monitor(c, m, s);
            if (rc) return rc;
        }
    }
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

int dft_flush_monitor(pc_ctx* c, DftMonitor& m, cudaStream_t s) {
    if (m.rows == 0) return PC_OK;
    dft_phase<<<(m.nf + 127) / 128, 128, 0, s>>>(m.d_state, m.d_rot, m.nf, m.rows, m.d_table);
    dim3 grd((m.npts + 255) / 256, m.nf);
    dft_flush<<<grd, 256, 0, s>>>(m.d_ring, m.npts, m.rows, m.d_table, m.nf, (float)m.dt, m.d_acc);
    c->launches += 2;
    m.rows = 0;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

}  // namespace pc
