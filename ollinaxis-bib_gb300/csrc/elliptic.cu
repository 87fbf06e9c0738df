// Elliptic initial data on the device: the WaveElliptic solver of
// src/elliptic/wave_elliptic.f90 and the scalar-pulse coefficients of
// src/matter/idata_scalarpulse.f90.
//
// WaveElliptic finds the stationary state of
//     du/dt = v,   dv/dt = lap(u) + S1 u + S5 u^5 - S0 - eta v
// with the same Berger-Oliger recursion, ICN/RK4 stages, Kreiss-Oliger
// dissipation, radiative boundary and refinement transfers as the evolution.
// One stage of one level is one launch of ``wave_stage_kernel`` over every
// point of the level.  A ghost point takes the source of its mirror image,
// which is what the reference's parity fill of sell_v gives.  The u-source
// of a ghost point is its own v.
// The residual of each iteration (RMS of sell_v over the level-0 interior)
// is reduced in a fixed order: per-block partial sums, then one block.
// ``EllCtl`` carries the stop condition on the device, so the host can queue
// batches of iterations that turn into no-ops once the solve has converged.
#include "ollin_kernels.h"

namespace ollin {

namespace {

constexpr int kWaveBX = 32, kWaveBY = 4, kWaveThreads = kWaveBX * kWaveBY;

__global__ void __launch_bounds__(kWaveThreads) wave_stage_kernel(const __grid_constant__ WaveArgs A) {
    __shared__ double red[kWaveThreads];
    if (A.skip && *A.skip) return;  // the same value for the whole grid
    const LevelGeom& G = A.G;
    const int g = G.g, nr = G.nr, nz = G.nz;
    const int i = 1 - g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - g + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    double res = 0.0;
    if (i <= nr && j <= nz) {
        const long ld = G.ld;
        const int mi = i < 1 ? 1 - i : i;
        const int mj = (G.eqsym && j < 1) ? 1 - j : j;
        const size_t o = (size_t)i + (size_t)j * ld, om = (size_t)mi + (size_t)mj * ld;
        const double* u = A.u_in + om;
        const double* v = A.v_in + om;
        const int pcr = pclass(mi, nr, g), pcz = pclass(mj, nz, g);
        const double cr1 = G.idr * (1.0 / 12.0), cz1 = G.idz * (1.0 / 12.0);
        const double cr2 = G.idr * G.idr * (1.0 / 12.0), cz2 = G.idz * G.idz * (1.0 / 12.0);
        // flat Laplacian in (r, z) with the axis term (wave_elliptic.f90:593-597)
        double s = (d2(u, 1, pcr, cr2) + d2(u, ld, pcz, cz2)) + d1(u, 1, pcr, cr1) * G.ircol[mi];
        const double uc = ld_(u);
        double u5 = uc * uc;
        u5 = u5 * u5;
        u5 = u5 * uc;
        s = s + ld_(A.S1 + om) * uc + ld_(A.S5 + om) * u5 - ld_(A.S0 + om);
        s = s - A.eta * ld_(v);
        // Kreiss-Oliger dissipation on v (dissipation.f90:196-211)
        const bool diss_r = (mi >= 4 - g && mi <= nr - 3), diss_z = (mj >= 4 - g && mj <= nz - 3);
        const double kd = A.kdiss * (1.0 / 20.0);
        if (diss_r && diss_z) {
            s = ko6rz_apply(v, ld, kd, s);
        } else {
            if (diss_r) s = s - kd * ko6(v, 1);
            if (diss_z) s = s - kd * ko6(v, ld);
        }
        // radiative boundary with unit speed and zero asymptotic value
        // (radbound(1.d0, 0.d0), radbound.f90:46-70)
        if (mi == nr || mj == nz) {
            const double r = G.rcol[mi], z = G.zrow[mj];
            const double rr = sqrt(r * r + z * z);
            s = -(r * d1(v, 1, pcr, cr1) + z * d1(v, ld, pcz, cz1) + (ld_(v) - 0.0)) / rr;
        }
        double su = ld_(A.v_in + o);  // sell_u = ell_v
        double sv = s;
        if (A.rk4) {
            if (A.iter == 1) {
                A.u_acc[o] = A.weight * su;
                A.v_acc[o] = A.weight * sv;
            } else if (A.iter < A.niter) {
                A.u_acc[o] = A.u_acc[o] + A.weight * su;
                A.v_acc[o] = A.v_acc[o] + A.weight * sv;
            } else {
                su = A.u_acc[o] + A.weight * su;
                sv = A.v_acc[o] + A.weight * sv;
            }
        }
        A.u_out[o] = ld_(A.u_p + o) + A.dtw * su;
        A.v_out[o] = ld_(A.v_p + o) + A.dtw * sv;
        if (i >= 1 && i <= nr - g && j >= 1 && j <= nz - g) res = sv * sv;
    }
    if (A.res_partial) {
        const int t = threadIdx.y * blockDim.x + threadIdx.x;
        red[t] = res;
        __syncthreads();
        for (int w = kWaveThreads / 2; w > 0; w >>= 1) {
            if (t < w) red[t] = red[t] + red[t + w];
            __syncthreads();
        }
        if (t == 0) A.res_partial[blockIdx.y * gridDim.x + blockIdx.x] = red[0];
    }
}

// wave_elliptic.f90:215-238: gres = sqrt(sum(sell_v^2)/(Nr*Nz)); then the
// loop condition of :206
__global__ void __launch_bounds__(256) wave_residual_kernel(const double* partial, int nparts, int nr, int nz, EllCtl* ctl) {
    __shared__ double red[256];
    if (ctl->done) return;
    const int t = threadIdx.x;
    double acc = 0.0;
    for (int k = t; k < nparts; k += 256) acc = acc + partial[k];
    red[t] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w) red[t] = red[t] + red[t + w];
        __syncthreads();
    }
    if (t == 0) {
        const int step = ctl->step + 1;
        const double gres = sqrt(red[0] / (double)(nr * nz));
        ctl->step = step;
        ctl->gres = gres;
        ctl->done = (step < ctl->miniter || (gres > ctl->eps && step < ctl->maxiter)) ? 0 : 1;
    }
}

// scalar_xi_r = diff1r(+1), scalar_xi_z = diff1z(+1) of scalar_phi at the
// interior points; the ghosts follow from the parity fill
__global__ void __launch_bounds__(128) pulse_xi_kernel(const __grid_constant__ PulseCoeffArgs a) {
    const LevelGeom& G = a.G;
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const long ld = G.ld;
    const size_t o = (size_t)i + (size_t)j * ld;
    const double* f = a.sphi + o;
    a.xir[o] = d1(f, 1, pclass(i, G.nr, G.g), G.idr * (1.0 / 12.0));
    a.xiz[o] = d1(f, ld, pclass(j, G.nz, G.g), G.idz * (1.0 / 12.0));
}

// idata_scalarpulse.f90:152-170 and potential.f90 at every point
__global__ void __launch_bounds__(128) pulse_coeff_kernel(const __grid_constant__ PulseCoeffArgs a) {
    const LevelGeom& G = a.G;
    const int g = G.g;
    const int i = 1 - g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - g + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const size_t o = (size_t)i + (size_t)j * G.ld;
    const double pi = 3.141592653589793;
    const double xr = a.xir[o], xz = a.xiz[o], ph = a.sphi[o];
    double V = 0.0;
    if (a.potential == 1) {
        V = 0.5 * (a.mass * a.mass) * (ph * ph);
    } else if (a.potential == 2) {
        const double p2 = ph * ph;
        V = 0.5 * (a.mass * a.mass) * p2 + 0.25 * a.lambda * (p2 * p2);
    }
    a.spi[o] = 0.0;
    a.S0[o] = 0.0;
    a.S1[o] = pi * (xr * xr + xz * xz);
    a.S5[o] = (a.potential == 0) ? 0.0 : 2.0 * pi * V;
}

}  // namespace

int wave_stage_blocks(const LevelGeom& G) {
    const int nx = (G.nr + G.g + kWaveBX - 1) / kWaveBX, ny = (G.nz + G.g + kWaveBY - 1) / kWaveBY;
    return nx * ny;
}

void launch_wave_stage(const WaveArgs& a, cudaStream_t s) {
    dim3 blk(kWaveBX, kWaveBY);
    dim3 grd((a.G.nr + a.G.g + kWaveBX - 1) / kWaveBX, (a.G.nz + a.G.g + kWaveBY - 1) / kWaveBY);
    wave_stage_kernel<<<grd, blk, 0, s>>>(a);
}

void launch_wave_residual(const double* partial, int nparts, int nr, int nz, EllCtl* ctl, cudaStream_t s) {
    wave_residual_kernel<<<1, 256, 0, s>>>(partial, nparts, nr, nz, ctl);
}

void launch_pulse_xi(const PulseCoeffArgs& a, cudaStream_t s) {
    dim3 blk(32, 4);
    dim3 grd((a.G.nr + blk.x - 1) / blk.x, (a.G.nz + blk.y - 1) / blk.y);
    pulse_xi_kernel<<<grd, blk, 0, s>>>(a);
}

void launch_pulse_coeffs(const PulseCoeffArgs& a, cudaStream_t s) {
    dim3 blk(32, 4);
    dim3 grd((a.G.nr + a.G.g + blk.x - 1) / blk.x, (a.G.nz + a.G.g + blk.y - 1) / blk.y);
    pulse_coeff_kernel<<<grd, blk, 0, s>>>(a);
}

}  // namespace ollin
