// Elliptic initial data on the device: the WaveElliptic solver of
// src/elliptic/wave_elliptic.f90, the SOR solver of
// src/elliptic/sor_elliptic.f90 and the scalar-pulse coefficients of
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

template <bool PHYS>
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
        const int ord = G.order;
        const int pcr = pclass_o(ord, mi, nr, g), pcz = pclass_o(ord, mj, nz, g);
        const double cr1 = c1_o(ord, G.idr), cz1 = c1_o(ord, G.idz);
        const double cr2 = c2_o(ord, G.idr), cz2 = c2_o(ord, G.idz);
        double s;
        if constexpr (!PHYS) {
            // flat Laplacian in (r, z) with the axis term (wave_elliptic.f90:593-597)
            s = (d2_o(ord, u, 1, pcr, cr2) + d2_o(ord, u, ld, pcz, cz2)) + d1_o(ord, u, 1, pcr, cr1) * G.ircol[mi];
        } else {
            // physical Laplacian of the conformal metric (wave_elliptic.f90:
            // 781-812); the hdet terms vanish (hdet = 1)
            const WavePhys& q = A.ph;
            const double ur = d1_o(ord, u, 1, pcr, cr1), uz = d1_o(ord, u, ld, pcz, cz1);
            const double urr = d2_o(ord, u, 1, pcr, cr2), uzz = d2_o(ord, u, ld, pcz, cz2);
            const double urz = d2rz_o(ord, u, ld, mi, mj, nr, nz, g, G.idr * G.idz);
            const double gA = q.gA[om], gB = q.gB[om], gC = q.gC[om];
            const double r = G.rcol[mi], rgC = r * gC;
            s = gA * urr + gB * uzz + ((2.0 * r) * gC) * urz;
            s = s + ur * q.P1[om] + uz * q.P2[om];
            s = s + (gA * ur) / r + gC * uz;
            s = s + 2.0 * (q.Drphi[om] * (gA * ur + rgC * uz) + q.Dzphi[om] * (gB * uz + rgC * ur));
            s = s / q.psi4[om];
        }
        const double uc = ld_(u);
        double u5 = uc * uc;
        u5 = u5 * u5;
        u5 = u5 * uc;
        s = s + ld_(A.S1 + om) * uc + ld_(A.S5 + om) * u5 - ld_(A.S0 + om);
        s = s - A.eta * ld_(v);
        // Kreiss-Oliger dissipation on v (dissipation.f90:196-211; order two
        // :121-135)
        if (ord == 2) {
            const bool diss_r = (mi >= 3 - g && mi <= nr - 2), diss_z = (mj >= 3 - g && mj <= nz - 2);
            const double kd = A.kdiss * (1.0 / 6.0);
            if (diss_r) s = s - kd * ko4(v, 1);
            if (diss_z) s = s - kd * ko4(v, ld);
        } else {
            const bool diss_r = (mi >= 4 - g && mi <= nr - 3), diss_z = (mj >= 4 - g && mj <= nz - 3);
            const double kd = A.kdiss * (1.0 / 20.0);
            if (diss_r && diss_z) {
                s = ko6rz_apply(v, ld, kd, s);
            } else {
                if (diss_r) s = s - kd * ko6(v, 1);
                if (diss_z) s = s - kd * ko6(v, ld);
            }
        }
        // radiative boundary with unit speed and zero asymptotic value
        // (radbound(1.d0, 0.d0), radbound.f90:46-70), also on the lower z
        // edge without equatorial symmetry
        if (mi == nr || mj == nz || (!G.eqsym && mj == 1 - g)) {
            const double r = G.rcol[mi], z = G.zrow[mj];
            const double rr = sqrt(r * r + z * z);
            s = -(r * d1_o(ord, v, 1, pcr, cr1) + z * d1_o(ord, v, ld, pcz, cz1) + (ld_(v) - 0.0)) / rr;
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
// interior points (without equatorial symmetry the lower rows too, one-sided
// in z); the other ghosts follow from the parity fill
__global__ void __launch_bounds__(128) pulse_xi_kernel(const __grid_constant__ PulseCoeffArgs a) {
    const LevelGeom& G = a.G;
    // on a grid off the axis the ghost columns too: diff1z covers them, while
    // diff1r leaves xi_r there unset (zero in data that start from zero)
    const int i = (G.axis ? 1 : 1 - G.g) + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = G.jlo + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const long ld = G.ld;
    const size_t o = (size_t)i + (size_t)j * ld;
    const double* f = a.sphi + o;
    const int ord = G.order;
    a.xir[o] = i < d1r_first(ord, G.g) ? 0.0 : d1_o(ord, f, 1, pclass_o(ord, i, G.nr, G.g), c1_o(ord, G.idr));
    a.xiz[o] = d1_o(ord, f, ld, pclass_o(ord, j, G.nz, G.g), c1_o(ord, G.idz));
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

// ---- SOR (sor_elliptic.f90:562-802) --------------------------------------
// Explicitly rounded operations throughout: the sweep and the boundary give
// the same bits as the sequential Fortran loops (the flat operator couples a
// point only to the other colour, so the order within a pass is immaterial).
__device__ __forceinline__ double mrn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double arn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double srn(double a, double b) { return __dsub_rn(a, b); }

constexpr int kSorBX = 32, kSorBY = 4, kSorThreads = kSorBX * kSorBY;

// e(i,j) = aux(i,j) + S5 u^4 (sor_elliptic.f90:632-636)
__global__ void __launch_bounds__(128) sor_e_kernel(LevelGeom G, double* e, const double* eaux, const double* S5,
                                                    const double* u, const int* skip) {
    if (skip && *skip) return;
    const int g = G.g;
    const int i = 2 - g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 2 - g + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr - 1 || j > G.nz - 1) return;
    const size_t o = (size_t)i + (size_t)j * G.ld;
    double u4 = mrn(u[o], u[o]);
    u4 = mrn(u4, u4);
    e[o] = arn(eaux[o], mrn(S5[o], u4));
}

// thread space: i over 2-g..Nr-1, jh over the points of the pass's parity in
// each column
__global__ void __launch_bounds__(kSorThreads) sor_pass_kernel(const __grid_constant__ SorPassArgs A) {
    __shared__ double red[kSorThreads];
    if (A.skip && *A.skip) return;
    const LevelGeom& G = A.G;
    const int g = G.g;
    const int i = 2 - g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int jh = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    // first j >= 2-g with (i + j) of the pass's parity
    int j = 2 - g;
    if (((i + j) & 1) != A.parity) ++j;
    j += 2 * jh;
    double res = 0.0;
    if (i <= G.nr - 1 && j <= G.nz - 1) {
        const long ld = G.ld;
        const size_t o = (size_t)i + (size_t)j * ld;
        double* u = A.u + o;
        const double ev = A.e[o];
        double r = mrn(A.ca[i], u[1]);
        r = arn(r, mrn(A.cb[i], u[-1]));
        r = arn(r, mrn(A.cc, u[ld]));
        r = arn(r, mrn(A.cc, u[-ld]));
        r = arn(r, mrn(ev, u[0]));
        r = srn(r, A.f[o]);
        res = mrn(r, r);
        u[0] = srn(u[0], __ddiv_rn(mrn(A.omega, r), ev));
    }
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    red[t] = res;
    __syncthreads();
    for (int w = kSorThreads / 2; w > 0; w >>= 1) {
        if (t < w) red[t] = red[t] + red[t + w];
        __syncthreads();
    }
    if (t == 0) A.partial[blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// fixed-order sum of n partials by the whole block
__device__ double block_sum(const double* partial, int n, double* red) {
    const int t = threadIdx.x;
    double acc = 0.0;
    for (int k = t; k < n; k += blockDim.x) acc = acc + partial[k];
    red[t] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (t < w) red[t] = red[t] + red[t + w];
        __syncthreads();
    }
    const double v = red[0];
    __syncthreads();
    return v;
}

// The Robin boundary of sor_elliptic.f90:698-756 is a recurrence along each
// outer edge: the point j of the r edge uses the new value at j-1.  Every
// other operand is known before the edge is swept, so the block first
// evaluates those in parallel into shared memory (the same operations in the
// same order), then one thread per edge runs the recurrence from shared
// memory (the r and z edges do not read each other's new values), and the
// block writes the edges back.  The corner follows from both edges.
__global__ void __launch_bounds__(1024) sor_finish_kernel(const __grid_constant__ SorFinishArgs A) {
    __shared__ double red[1024];
    extern __shared__ double edge[];
    EllCtl* ctl = A.ctl;
    if (ctl->done) return;
    const LevelGeom& G = A.G;
    const int g = G.g, nr = G.nr, nz = G.nz;
    const long ld = G.ld;
    double* u = A.u;
    auto U = [&](int i, int j) -> double& { return u[(size_t)i + (size_t)j * ld]; };
    const double npts = (double)((nr + g) * (nz + g));  // imax*jmax
    // anorm after pass 1 is sqrt(sum1/N); pass 2 keeps adding to that value
    const double s1 = block_sum(A.partial1, A.nparts, red);
    const double s2 = block_sum(A.partial2, A.nparts, red);
    const double anorm1 = sqrt(s1 / npts);
    const double ganorm = sqrt((anorm1 + s2) / npts);
    if (A.robin) {
        const int nj = nz + g, ni = nr + g;  // edge arrays indexed by j+g-1 / i+g-1
        double* Pr = edge;                 // uinf + 0.5 cr (4 u(Nr-1,j) - u(Nr-2,j))
        double* Qr = Pr + nj;              // old u(Nr, j+1)
        double* Hr = Qr + nj;              // 0.5 z(j)/dz
        double* Pz = Hr + nj;              // uinf + 0.5 cz (4 u(i,Nz-1) - u(i,Nz-2))
        double* Qz = Pz + ni;              // old u(i+1, Nz)
        double* Hz = Qz + ni;              // 0.5 r(i)/dr
        // without equatorial symmetry the lower z edge as well (:724-736)
        const bool lower = !G.eqsym;
        double* Pl = Hz + ni;              // uinf - 0.5 czl (4 u(i,2-g) - u(i,3-g))
        double* Ql = Pl + ni;              // old u(i+1, 1-g)
        const double crn = G.rcol[nr] / G.dr, czn = G.zrow[nz] / G.dz, czl = G.zrow[1 - g] / G.dz;
        for (int j = 2 - g + (int)threadIdx.x; j <= nz - 1; j += blockDim.x) {
            const int k = j + g - 1;
            Pr[k] = arn(A.uinf, mrn(mrn(0.5, crn), srn(mrn(4.0, U(nr - 1, j)), U(nr - 2, j))));
            Qr[k] = U(nr, j + 1);
            Hr[k] = mrn(0.5, G.zrow[j] / G.dz);
        }
        for (int i = 2 - g + (int)threadIdx.x; i <= nr - 1; i += blockDim.x) {
            const int k = i + g - 1;
            Pz[k] = arn(A.uinf, mrn(mrn(0.5, czn), srn(mrn(4.0, U(i, nz - 1)), U(i, nz - 2))));
            Qz[k] = U(i + 1, nz);
            Hz[k] = mrn(0.5, G.rcol[i] / G.dr);
            if (lower) {
                Pl[k] = srn(A.uinf, mrn(mrn(0.5, czl), srn(mrn(4.0, U(i, 2 - g)), U(i, 3 - g))));
                Ql[k] = U(i + 1, 1 - g);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {  // r edge, j upwards
            const double den = arn(1.0, mrn(1.5, crn));
            double prev = U(nr, 1 - g);
            for (int k = 1; k <= nz - 2 + g; ++k) {  // j = 2-g .. nz-1
                prev = __ddiv_rn(srn(Pr[k], mrn(Hr[k], srn(Qr[k], prev))), den);
                Pr[k] = prev;
            }
        } else if (threadIdx.x == 32) {  // upper z edge, i outwards
            const double den = arn(1.0, mrn(1.5, czn));
            double prev = U(1 - g, nz);
            for (int k = 1; k <= nr - 2 + g; ++k) {  // i = 2-g .. nr-1
                prev = __ddiv_rn(srn(Pz[k], mrn(Hz[k], srn(Qz[k], prev))), den);
                Pz[k] = prev;
            }
        } else if (threadIdx.x == 64 && lower) {  // lower z edge, i outwards
            const double den = srn(1.0, mrn(1.5, czl));
            double prev = U(1 - g, 1 - g);
            for (int k = 1; k <= nr - 2 + g; ++k) {  // i = 2-g .. nr-1
                prev = __ddiv_rn(srn(Pl[k], mrn(Hz[k], srn(Ql[k], prev))), den);
                Pl[k] = prev;
            }
        }
        __syncthreads();
        for (int j = 2 - g + (int)threadIdx.x; j <= nz - 1; j += blockDim.x) U(nr, j) = Pr[j + g - 1];
        for (int i = 2 - g + (int)threadIdx.x; i <= nr - 1; i += blockDim.x) {
            U(i, nz) = Pz[i + g - 1];
            if (lower) U(i, 1 - g) = Pl[i + g - 1];
        }
        __syncthreads();
        if (threadIdx.x == 0) {  // upper corner (:738-745)
            double v = arn(A.uinf, mrn(mrn(0.5, crn), srn(mrn(4.0, U(nr - 1, nz)), U(nr - 2, nz))));
            v = arn(v, mrn(mrn(0.5, czn), srn(mrn(4.0, U(nr, nz - 1)), U(nr, nz - 2))));
            U(nr, nz) = __ddiv_rn(v, arn(1.0, mrn(1.5, arn(crn, czn))));
            if (lower) {  // lower corner (:747-756)
                double w = arn(A.uinf, mrn(mrn(0.5, crn), srn(mrn(4.0, U(nr - 1, 1 - g)), U(nr - 2, 1 - g))));
                w = srn(w, mrn(mrn(0.5, czl), srn(mrn(4.0, U(nr, 2 - g)), U(nr, 3 - g))));
                U(nr, 1 - g) = __ddiv_rn(w, arn(1.0, mrn(1.5, srn(crn, czl))));
            }
        }
    }
    __syncthreads();
    // parity fill: axis first over all rows, then the equator (:772-784),
    // on a grid that owns them (a refinement box off the axis or the
    // equator keeps its interpolated ghosts as Dirichlet values)
    if (G.axis)
        for (int j = 1 - g + (int)threadIdx.x; j <= nz; j += blockDim.x)
            for (int i = 1; i <= g; ++i) U(1 - i, j) = U(i, j);
    __syncthreads();
    if (G.equator)
        for (int i = 1 - g + (int)threadIdx.x; i <= nr; i += blockDim.x)
            for (int j = 1; j <= g; ++j) U(i, 1 - j) = U(i, j);
    if (threadIdx.x == 0) {
        const int step = ctl->step + 1;
        ctl->step = step;
        ctl->gres = ganorm;
        ctl->done = (ganorm < ctl->eps || step >= ctl->maxiter) ? 1 : 0;
    }
}

// ---- maximal slicing (maximalslicing.f90) -----------------------------------
constexpr int kMaxBX = 32, kMaxBY = 4, kMaxThreads = kMaxBX * kMaxBY;

// Coefficients of the physical Laplacian and the source S1 at every point
// (MaxCoeffArgs); per-block maxima of the light speeds sqrt|g^ii/psi4| for
// the wave solver's time step (wave_elliptic.f90:193-263).  A derivative at
// a ghost point is the parity image of the derivative at the mirror point,
// as the symmetry fill of derivatives.f90:91-99 and :212-216 leaves it: the
// r derivative changes sign across the axis for an even function and takes
// the function's z parity across the equator, and the other way round for
// the z derivative.
__global__ void __launch_bounds__(kMaxThreads) max_coeff_kernel(const __grid_constant__ MaxCoeffArgs A) {
    __shared__ double red[2][kMaxThreads];
    const LevelGeom& G = A.G;
    const int g = G.g, nr = G.nr, nz = G.nz;
    const int i = 1 - g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - g + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    double vr = 0.0, vz = 0.0;
    if (i <= nr && j <= nz) {
        const long ld = G.ld;
        // a ghost column of a grid off the axis keeps r derivatives of zero
        // (diff1r leaves them unset there); ghost rows of a grid that does
        // not own the equator take the one-sided z stencils
        const int ord = G.order;
        const bool gr = G.axis && i < 1, gz = G.equator && j < 1, r0 = !G.axis && i < d1r_first(ord, g);
        const int mi = gr ? 1 - i : i, mj = gz ? 1 - j : j;
        const size_t o = (size_t)i + (size_t)j * ld, om = (size_t)mi + (size_t)mj * ld;
        // the arrays the derivatives are taken from: the live ones, or after
        // syncboxes the state before the copy (or the partner's, at a
        // copied point: interior stencils there)
        const double* src[5] = {A.gA, A.gB, A.gC, A.chi, A.phi};
        size_t os = om;
        long lds = ld;
        bool xin = false;
        if (A.smap) {
            const int m = A.smap[om];
            const int pk = m >= 0 ? m >> kPartnerShift : 0;
            for (int k = 0; k < 5; ++k) src[k] = m >= 0 ? A.xb[pk][k] : A.xa[k];
            if (m >= 0) { os = (size_t)(m & kPartnerOffset); lds = A.xb_ld[pk]; xin = true; }
        }
        const int pcr = xin ? 0 : pclass_o(ord, mi, nr, g), pcz = xin ? 0 : pclass_o(ord, mj, nz, g);
        const double cr1 = c1_o(ord, G.idr), cz1 = c1_o(ord, G.idz);
        auto d1 = [ord](const double* f, long st, int k, double c) { return d1_o(ord, f, st, k, c); };
        // parities: g_A, g_B, phi, chi even in r and z; g_C even in r, odd in z
        const double er = gr ? -1.0 : 1.0;  // r derivative of an r-even function
        const double ez = gz ? -1.0 : 1.0;  // z derivative of a z-even function
        const double DrgA = r0 ? 0.0 : d1(src[0] + os, 1, pcr, cr1) * er;
        const double DzgB = d1(src[1] + os, lds, pcz, cz1) * ez;
        const double DrgC = r0 ? 0.0 : d1(src[2] + os, 1, pcr, cr1) * er * (gz ? -1.0 : 1.0);
        const double DzgC = d1(src[2] + os, lds, pcz, cz1);
        const double r = G.rcol[i], gC = A.gC[o];
        A.P1[o] = DrgA + r * DzgC;
        A.P2[o] = (DzgB + r * DrgC) + gC;
        double Drphi, Dzphi, psi4;
        if (A.t0) {
            Drphi = r0 ? 0.0 : d1(src[4] + os, 1, pcr, cr1) * er;
            Dzphi = d1(src[4] + os, lds, pcz, cz1) * ez;
            const double p = exp(A.phi[o]);
            psi4 = (p * p) * (p * p);
        } else {
            const double chm = src[3][os];
            Drphi = r0 ? 0.0 : (-(d1(src[3] + os, 1, pcr, cr1) * er) / chm) * 0.5;
            Dzphi = (-(d1(src[3] + os, lds, pcz, cz1) * ez) / chm) * 0.5;
            const double p = exp(-log(A.chi[o]) * 0.5);
            psi4 = (p * p) * (p * p);
        }
        A.Drphi[o] = Drphi;
        A.Dzphi[o] = Dzphi;
        A.psi4[o] = psi4;
        const double tk = A.trK[om];
        double s1 = -(A.KT2[om] + (1.0 / 3.0) * (tk * tk));
        if (A.rhos) s1 = s1 - 4.0 * 3.141592653589793 * A.rhos[om];
        A.S1[o] = s1;
        vr = sqrt(fabs(A.gA[o] / psi4));
        vz = sqrt(fabs(A.gB[o] / psi4));
    }
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    red[0][t] = vr;
    red[1][t] = vz;
    __syncthreads();
    for (int w = kMaxThreads / 2; w > 0; w >>= 1) {
        if (t < w) {
            red[0][t] = fmax(red[0][t], red[0][t + w]);
            red[1][t] = fmax(red[1][t], red[1][t + w]);
        }
        __syncthreads();
    }
    const int b = blockIdx.y * gridDim.x + blockIdx.x;
    if (t == 0) { A.vmax[2 * b] = red[0][0]; A.vmax[2 * b + 1] = red[1][0]; }
}

// SOR stencil of the physical Laplacian at every point, in the expression
// order of sor_elliptic.f90:168-262 / :371-448 (explicitly rounded)
__global__ void __launch_bounds__(128) sor_coeff_kernel(const __grid_constant__ SorCoeffArgs A) {
    const LevelGeom& G = A.G;
    const int g = G.g;
    const int i = 1 - g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - g + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const size_t o = (size_t)i + (size_t)j * G.ld;
    const WavePhys& q = A.ph;
    const double dr = G.dr, dz = G.dz, r = G.rcol[i];
    const double gA = q.gA[o], gB = q.gB[o], gC = q.gC[o], ps = q.psi4[o];
    const double Drp = q.Drphi[o], Dzp = q.Dzphi[o];
    auto dv = [](double x, double y) { return __ddiv_rn(x, y); };
    double a = dv(mrn(gA, arn(dv(1.0, dr), dv(0.5, r))), dr);
    double b = dv(mrn(gA, srn(dv(1.0, dr), dv(0.5, r))), dr);
    double c = dv(gB, mrn(dz, dz));
    double d = dv(gB, mrn(dz, dz));
    double e = mrn(-2.0, arn(dv(gA, mrn(dr, dr)), dv(gB, mrn(dz, dz))));
    const double hr = mrn(mrn(0.5, r), gC);
    const double diag = A.fine ? dv(dv(hr, dr), dz) : dv(hr, mrn(dr, dz));
    double cg = diag, ch = diag, ci = -diag, cj = -diag;
    const double t1 = dv(mrn(0.5, q.P1[o]), dr), t2 = dv(mrn(0.5, q.P2[o]), dz);
    a = arn(a, t1); b = srn(b, t1);
    c = arn(c, t2); d = srn(d, t2);
    const double t3 = dv(mrn(0.5, gC), dz);
    c = arn(c, t3); d = srn(d, t3);
    const double rgC = mrn(r, gC);
    const double t4 = dv(arn(mrn(gA, Drp), mrn(rgC, Dzp)), dr);
    const double t5 = dv(arn(mrn(gB, Dzp), mrn(rgC, Drp)), dz);
    a = arn(a, t4); b = srn(b, t4);
    c = arn(c, t5); d = srn(d, t5);
    A.a[o] = dv(a, ps); A.b[o] = dv(b, ps); A.c[o] = dv(c, ps); A.d[o] = dv(d, ps);
    A.e[o] = arn(dv(e, ps), A.S1[o]);
    cg = dv(cg, ps); ch = dv(ch, ps); ci = dv(ci, ps); cj = dv(cj, ps);
    A.cg[o] = cg; A.ch[o] = ch; A.ci[o] = ci; A.cj[o] = cj;
    if (cg != 0.0 || ch != 0.0 || ci != 0.0 || cj != 0.0) atomicOr(A.diag_nonzero, 1ull);
}

// residual of the nine-point stencil at one point, in the order of
// sor_elliptic.f90:660-666, and the update of u
__device__ __forceinline__ double sor_phys_update(const SorPhysPassArgs& A, size_t o, long ld, bool diag) {
    double* u = A.u + o;
    const double ev = A.e[o];
    double r = mrn(A.a[o], u[1]);
    r = arn(r, mrn(A.b[o], u[-1]));
    r = arn(r, mrn(A.c[o], u[ld]));
    r = arn(r, mrn(A.d[o], u[-ld]));
    if (diag) {
        r = arn(r, mrn(A.cg[o], u[1 + ld]));
        r = arn(r, mrn(A.ch[o], u[-1 - ld]));
        r = arn(r, mrn(A.ci[o], u[1 - ld]));
        r = arn(r, mrn(A.cj[o], u[-1 + ld]));
    }
    r = arn(r, mrn(ev, u[0]));
    r = srn(r, A.f[o]);
    u[0] = srn(u[0], __ddiv_rn(mrn(A.omega, r), ev));
    return mrn(r, r);
}

// A pass when every diagonal coefficient is zero: the points of one colour
// are then independent, as for the flat Laplacian
__global__ void __launch_bounds__(kSorThreads) sor_phys_pass_kernel(const __grid_constant__ SorPhysPassArgs A) {
    __shared__ double red[kSorThreads];
    if (A.skip && *A.skip) return;
    const LevelGeom& G = A.G;
    const int g = G.g;
    const int i = 2 - g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int jh = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    int j = 2 - g;
    if (((i + j) & 1) != A.parity) ++j;
    j += 2 * jh;
    double res = 0.0;
    if (i <= G.nr - 1 && j <= G.nz - 1) res = sor_phys_update(A, (size_t)i + (size_t)j * G.ld, G.ld, false);
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    red[t] = res;
    __syncthreads();
    for (int w = kSorThreads / 2; w > 0; w >>= 1) {
        if (t < w) red[t] = red[t] + red[t + w];
        __syncthreads();
    }
    if (t == 0) A.partial[blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// A pass with nonzero diagonal coefficients: they couple a point to the
// points of its own colour in the neighbouring columns, which the loop of
// sor_elliptic.f90:648-676 (i outer) has already updated (i-1) or not yet
// (i+1).  One block sweeps the columns in that order; within a column the
// points are independent.
constexpr int kSeqThreads = 1024;
__global__ void __launch_bounds__(kSeqThreads) sor_phys_pass_seq_kernel(const __grid_constant__ SorPhysPassArgs A) {
    __shared__ double red[kSeqThreads];
    if (A.skip && *A.skip) return;
    const LevelGeom& G = A.G;
    const int g = G.g;
    const long ld = G.ld;
    double res = 0.0;
    for (int i = 2 - g; i <= G.nr - 1; ++i) {
        int j0 = 2 - g;
        if (((i + j0) & 1) != A.parity) ++j0;
        for (int j = j0 + 2 * (int)threadIdx.x; j <= G.nz - 1; j += 2 * kSeqThreads)
            res = res + sor_phys_update(A, (size_t)i + (size_t)j * ld, ld, true);
        __syncthreads();
    }
    const int t = threadIdx.x;
    red[t] = res;
    __syncthreads();
    for (int w = kSeqThreads / 2; w > 0; w >>= 1) {
        if (t < w) red[t] = red[t] + red[t + w];
        __syncthreads();
    }
    if (t == 0) A.partial[0] = red[0];
}

// out = c + x at every point
__global__ void add_kernel(LevelGeom G, double* out, double c, const double* x) {
    const int g = G.g;
    const int i = 1 - g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - g + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const size_t o = (size_t)i + (size_t)j * G.ld;
    out[o] = arn(c, x[o]);
}

// ---- mixed-precision solve of the SOR discretisation --------------------
// (FP64 residual and update here; the FP32 correction solve is in
// multigrid.cu)
// Unknowns u(i,j), 1 <= i <= Nr, 1 <= j <= Nz; ghosts mirror the first
// interior points (u(1-k,j) = u(k,j), u(i,1-k) = u(i,k)).  Equations:
//   interior  a_i u(i+1,j) + b_i u(i-1,j) + c (u(i,j+1) + u(i,j-1)) + e u - f = 0
//   r edge    (1+1.5cr) u(Nr,j) - uinf - 0.5cr(4u(Nr-1,j) - u(Nr-2,j))
//             + 0.5cz_j (u(Nr,j+1) - u(Nr,j-1)) = 0           (and the z edge)
//   corner    (1+1.5(cr+cz)) u - uinf - 0.5cr(..) - 0.5cz(..) = 0
// which is the fixed point of sor_elliptic.f90 (sweep, Robin rows, parity).
constexpr int kMixBX = 32, kMixBY = 4, kMixThreads = kMixBX * kMixBY;

__device__ __forceinline__ int mir(int k) { return k < 1 ? 1 - k : k; }

// The unknowns of a level's system: i from 1 on a grid that owns the axis
// (mirrored ghosts), from 2-ghost on a refinement box off it, where the
// outermost ghost column is the Dirichlet row from the parent, as SOR sweeps
// them (sor_elliptic.f90:648); likewise in z.  The upper rows nr, nz are
// Robin rows on the coarse problem and Dirichlet rows otherwise.
// Without equatorial symmetry the coarse problem's lowest row j = 1-ghost is a
// Robin row (sor_elliptic.f90:724-756), an unknown too.
__device__ __forceinline__ int mix_ilo(const LevelGeom& G) { return G.axis ? 1 : 2 - G.g; }
__device__ __forceinline__ int mix_jlo(const LevelGeom& G, int robin) {
    return G.equator ? 1 : (robin ? 1 - G.g : 2 - G.g);
}
// element (p, q) of a level array, mirrored across the axis / equator where
// the grid owns them
__device__ __forceinline__ size_t mix_at(const LevelGeom& G, int p, int q) {
    return (size_t)(G.axis ? mir(p) : p) + (size_t)(G.equator ? mir(q) : q) * (size_t)G.ld;
}

__device__ __forceinline__ void block_partial(double v, double* out) {
    __shared__ double red[kMixThreads];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    red[t] = v;
    __syncthreads();
    for (int w = kMixThreads / 2; w > 0; w >>= 1) {
        if (t < w) red[t] = red[t] + red[t + w];
        __syncthreads();
    }
    if (t == 0) out[blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// A sum of products c*u kept as an unevaluated pair (s, e): each product's
// rounding error from an FMA and each addition's from TwoSum (Knuth; Ogita,
// Rump and Oishi's Dot2), so the rounded total is good to about one unit of
// its own last place however much the terms cancel.  With EXACT false it is
// the plain FP64 sum.
template <bool EXACT>
struct RowSum {
    double s = 0.0, e = 0.0;
    __device__ __forceinline__ void prod(double c, double u) {
        if constexpr (EXACT) {
            const double p = __dmul_rn(c, u);
            const double ep = __fma_rn(c, u, -p);
            add_exact(p);
            e = __dadd_rn(e, ep);
        } else {
            s = s + c * u;
        }
    }
    __device__ __forceinline__ void add(double x) {
        if constexpr (EXACT) add_exact(x);
        else s = s + x;
    }
    __device__ __forceinline__ void add_exact(double x) {
        const double t = __dadd_rn(s, x);
        const double bb = __dsub_rn(t, s);
        const double err = __dadd_rn(__dsub_rn(s, __dsub_rn(t, bb)), __dsub_rn(x, bb));
        s = t;
        e = __dadd_rn(e, err);
    }
    __device__ __forceinline__ double value() const { return EXACT ? __dadd_rn(s, e) : s; }
};

// R(u) of the equation at unknown (i, j): the interior nine- or five-point
// row, or (robin) the Robin row.  The residual (EXACT) sums the products of
// the FP64 coefficients and unknowns without rounding loss, so the
// refinement converges to the FP64 solution of the system itself rather
// than to the rounding floor of its rows (about |e| ulp(u)); the operator
// applied to a correction (!EXACT) drops the data terms f and uinf and sums
// plainly.  Returns false on a Dirichlet row.
template <bool EXACT, typename UF>
__device__ __forceinline__ bool mix_row(const MixArgs& A, const UF& U, int i, int j, size_t o, double& R,
                                        bool& interior) {
    const LevelGeom& G = A.G;
    const int nr = G.nr, nz = G.nz;
    const bool low = A.robin && !G.equator && j == 1 - G.g;  // the lower Robin row
    interior = i <= nr - 1 && j <= nz - 1 && !low;  // and i >= mix_ilo, j >= mix_jlo (the callers' range)
    RowSum<EXACT> acc;
    if (interior) {
        if (!A.pa) {
            acc.prod(A.ca[i], U(i + 1, j));
            acc.prod(A.cb[i], U(i - 1, j));
            acc.prod(A.cc, U(i, j + 1));
            acc.prod(A.cc, U(i, j - 1));
        } else {
            acc.prod(A.pa[o], U(i + 1, j));
            acc.prod(A.pb[o], U(i - 1, j));
            acc.prod(A.pc[o], U(i, j + 1));
            acc.prod(A.pd[o], U(i, j - 1));
            acc.prod(A.pg[o], U(i + 1, j + 1));
            acc.prod(A.ph[o], U(i - 1, j - 1));
            acc.prod(A.pi[o], U(i + 1, j - 1));
            acc.prod(A.pj[o], U(i - 1, j + 1));
        }
        acc.prod(A.e64[o], U(i, j));
        if (EXACT) acc.add(-A.f64[o]);
        R = acc.value();
        return true;
    }
    if (!A.robin) return false;
    // (1 + 1.5 (cr + cz)) u - uinf - cr/2 (4 u_1 - u_2) - cz/2 (4 u_1 - u_2)
    // along each outward direction; a centred difference along the edge; on
    // the lower z edge the outward direction is -z (cz < 0 there)
    const double cr = G.rcol[i] / G.dr, cz = G.zrow[j] / G.dz;
    const double hr = 0.5 * cr, hz = 0.5 * cz;
    if (low && i == nr) {
        acc.prod(1.0 + 1.5 * (cr - cz), U(i, j));
        acc.prod(-4.0 * hr, U(i - 1, j));
        acc.prod(hr, U(i - 2, j));
        acc.prod(4.0 * hz, U(i, j + 1));
        acc.prod(-hz, U(i, j + 2));
    } else if (low) {
        acc.prod(1.0 - 1.5 * cz, U(i, j));
        acc.prod(4.0 * hz, U(i, j + 1));
        acc.prod(-hz, U(i, j + 2));
        acc.prod(hr, U(i + 1, j));
        acc.prod(-hr, U(i - 1, j));
    } else if (i == nr && j == nz) {
        acc.prod(1.0 + 1.5 * (cr + cz), U(i, j));
        acc.prod(-4.0 * hr, U(i - 1, j));
        acc.prod(hr, U(i - 2, j));
        acc.prod(-4.0 * hz, U(i, j - 1));
        acc.prod(hz, U(i, j - 2));
    } else if (i == nr) {
        acc.prod(1.0 + 1.5 * cr, U(i, j));
        acc.prod(-4.0 * hr, U(i - 1, j));
        acc.prod(hr, U(i - 2, j));
        acc.prod(hz, U(i, j + 1));
        acc.prod(-hz, U(i, j - 1));
    } else {
        acc.prod(1.0 + 1.5 * cz, U(i, j));
        acc.prod(-4.0 * hz, U(i, j - 1));
        acc.prod(hz, U(i, j - 2));
        acc.prod(hr, U(i + 1, j));
        acc.prod(-hr, U(i - 1, j));
    }
    if (EXACT) acc.add(-A.uinf);
    R = acc.value();
    return true;
}

// FP64 residual r = -R(u) at every unknown (zero on Dirichlet rows): into r64
// when set, and for the FP32 correction solve its FP32 copy with d = 0 (else
// d64 = 0); per-block sums over the interior equations of r^2 (into
// partial[b]) and of (e u)^2, the scale of the equation (partial[nblocks+b]),
// and over the Robin rows of r^2 (partial[2 nblocks+b]).
__global__ void __launch_bounds__(kMixThreads) mix_resid_kernel(const __grid_constant__ MixArgs A) {
    const LevelGeom& G = A.G;
    const long ld = G.ld;
    const int i = mix_ilo(G) + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = mix_jlo(G, A.robin) + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    double sq = 0.0, sc = 0.0, sb = 0.0;
    (void)ld;
    if (i <= G.nr && j <= G.nz) {
        auto U = [&](int p, int q) { return A.u[mix_at(G, p, q)]; };
        const size_t o = (size_t)i + (size_t)j * ld;
        double R = 0.0, r = 0.0;
        bool interior;
        if (mix_row<true>(A, U, i, j, o, R, interior)) r = -R;
        if (interior) {
            sq = r * r;
            const double eu = A.e64[o] * U(i, j);
            sc = eu * eu;
        } else {
            sb = r * r;
        }
        if (A.r64) A.r64[o] = r;
        if (A.d64) {
            A.d64[o] = 0.0;
        } else {
            A.r32[o] = (float)r;
            A.d[o] = 0.0f;
        }
    }
    block_partial(sq, A.partial);
    block_partial(sc, A.partial + gridDim.x * gridDim.y);
    block_partial(sb, A.partial + 2 * gridDim.x * gridDim.y);
}

// ---- Krylov acceleration of the multigrid corrections (Orthomin) ---------
// The multigrid correction z of a refinement becomes a search direction: q =
// A z is made orthogonal to the last few stored A-images, z follows with the
// same coefficients, and u moves by the alpha that minimises |r - alpha q|.
// The residual norm then never grows, even where the multigrid cycle alone
// diverges (a positive zeroth-order coefficient, the Helmholtz sign, on the
// coarse grids).

// z64 = the correction (widened from FP32 when the solve ran in FP32);
// q = A z64 (homogeneous rows, zero on Dirichlet rows)
__global__ void __launch_bounds__(kMixThreads) mix_apply_kernel(const __grid_constant__ MixArgs A, double* z64,
                                                                 double* q) {
    const LevelGeom& G = A.G;
    const long ld = G.ld;
    const int i = mix_ilo(G) + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = mix_jlo(G, A.robin) + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    auto Z = [&](int p, int qq) {
        // the correction is zero on a Dirichlet row (left zero by the solve)
        const size_t oo = mix_at(G, p, qq);
        return A.d64 ? A.d64[oo] : (double)A.d[oo];
    };
    const size_t o = (size_t)i + (size_t)j * ld;
    double R = 0.0;
    bool interior;
    const bool row = mix_row<false>(A, Z, i, j, o, R, interior);
    z64[o] = row ? Z(i, j) : 0.0;
    q[o] = row ? R : 0.0;
}

// per-block sums of x * y[k] over the unknowns, k < n (partial[k*nblocks+b])
__global__ void __launch_bounds__(kMixThreads) mix_dots_kernel(LevelGeom G, int robin, const double* x, OrthoVecs Y,
                                                                int n, double* partial) {
    const int i = mix_ilo(G) + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = mix_jlo(G, robin) + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const bool in = i <= G.nr && j <= G.nz;
    const size_t o = in ? (size_t)i + (size_t)j * G.ld : 0;
    const double xv = in ? x[o] : 0.0;
    const int nb = gridDim.x * gridDim.y;
    for (int k = 0; k < n; ++k) block_partial(in ? xv * Y.v[k][o] : 0.0, partial + (size_t)k * nb);
}

// z -= sum_k beta_k Z_k, q -= sum_k beta_k Q_k
__global__ void __launch_bounds__(kMixThreads) mix_orth_kernel(LevelGeom G, int robin, double* z, double* q,
                                                                OrthoVecs Zs, OrthoVecs Qs, OrthoCoef beta, int n) {
    const int i = mix_ilo(G) + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = mix_jlo(G, robin) + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const size_t o = (size_t)i + (size_t)j * G.ld;
    double zv = z[o], qv = q[o];
    for (int k = 0; k < n; ++k) {
        zv = zv - beta.c[k] * Zs.v[k][o];
        qv = qv - beta.c[k] * Qs.v[k][o];
    }
    z[o] = zv;
    q[o] = qv;
}

// u += alpha z at the unknowns that are not Dirichlet rows
__global__ void __launch_bounds__(kMixThreads) mix_step_kernel(LevelGeom G, int robin, double* u, const double* z,
                                                                double alpha) {
    const int i = mix_ilo(G) + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = mix_jlo(G, robin) + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int lim_r = robin ? G.nr : G.nr - 1, lim_z = robin ? G.nz : G.nz - 1;
    if (i > lim_r || j > lim_z) return;
    const size_t o = (size_t)i + (size_t)j * G.ld;
    u[o] = u[o] + alpha * z[o];
}

}  // namespace

// the mixed kernels' blocks over a level's unknowns
static dim3 mix_grid(const LevelGeom& G, int robin) {
    const int ni = G.nr - (G.axis ? 1 : 2 - G.g) + 1;
    const int nj = G.nz - (G.equator ? 1 : (robin ? 1 - G.g : 2 - G.g)) + 1;
    return dim3((ni + kMixBX - 1) / kMixBX, (nj + kMixBY - 1) / kMixBY);
}

int mix_blocks(const LevelGeom& G, int robin) {
    const dim3 b = mix_grid(G, robin);
    const int nx = (int)b.x, ny = (int)b.y;
    return nx * ny;
}

void launch_mix_resid(const MixArgs& a, cudaStream_t s) {
    dim3 blk(kMixBX, kMixBY);
    dim3 grd = mix_grid(a.G, a.robin);
    mix_resid_kernel<<<grd, blk, 0, s>>>(a);
}

void launch_mix_apply(const MixArgs& a, double* z64, double* q, cudaStream_t s) {
    dim3 blk(kMixBX, kMixBY);
    dim3 grd = mix_grid(a.G, a.robin);
    mix_apply_kernel<<<grd, blk, 0, s>>>(a, z64, q);
}

void launch_mix_dots(const LevelGeom& G, int robin, const double* x, const OrthoVecs& y, int n, double* partial,
                     cudaStream_t s) {
    dim3 blk(kMixBX, kMixBY);
    dim3 grd = mix_grid(G, robin);
    mix_dots_kernel<<<grd, blk, 0, s>>>(G, robin, x, y, n, partial);
}

void launch_mix_orth(const LevelGeom& G, int robin, double* z, double* q, const OrthoVecs& Zs, const OrthoVecs& Qs,
                     const OrthoCoef& beta, int n, cudaStream_t s) {
    dim3 blk(kMixBX, kMixBY);
    dim3 grd = mix_grid(G, robin);
    mix_orth_kernel<<<grd, blk, 0, s>>>(G, robin, z, q, Zs, Qs, beta, n);
}


void launch_mix_step(const LevelGeom& G, int robin, double* u, const double* z, double alpha, cudaStream_t s) {
    dim3 blk(kMixBX, kMixBY);
    dim3 grd = mix_grid(G, robin);
    mix_step_kernel<<<grd, blk, 0, s>>>(G, robin, u, z, alpha);
}

void launch_sor_e(const LevelGeom& G, double* e, const double* eaux, const double* S5, const double* u,
                  const int* skip, cudaStream_t s) {
    dim3 blk(32, 4);
    dim3 grd((G.nr + G.g - 2 + blk.x - 1) / blk.x, (G.nz + G.g - 2 + blk.y - 1) / blk.y);
    sor_e_kernel<<<grd, blk, 0, s>>>(G, e, eaux, S5, u, skip);
}

int sor_pass_blocks(const LevelGeom& G) {
    const int ni = G.nr + G.g - 2, nj = (G.nz + G.g - 2 + 1) / 2;
    return ((ni + kSorBX - 1) / kSorBX) * ((nj + kSorBY - 1) / kSorBY);
}

void launch_sor_pass(const SorPassArgs& a, cudaStream_t s) {
    const int ni = a.G.nr + a.G.g - 2, nj = (a.G.nz + a.G.g - 2 + 1) / 2;
    dim3 blk(kSorBX, kSorBY);
    dim3 grd((ni + kSorBX - 1) / kSorBX, (nj + kSorBY - 1) / kSorBY);
    sor_pass_kernel<<<grd, blk, 0, s>>>(a);
}

size_t sor_finish_smem(const LevelGeom& G) {
    return (size_t)(3 * (G.nz + G.g) + (G.eqsym ? 3 : 5) * (G.nr + G.g)) * sizeof(double);
}

int launch_sor_finish(const SorFinishArgs& a, cudaStream_t s) {
    const size_t smem = a.robin ? sor_finish_smem(a.G) : 0;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(sor_finish_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 1;
    sor_finish_kernel<<<1, 1024, smem, s>>>(a);
    return 0;
}

void launch_add(const LevelGeom& G, double* out, double c, const double* x, cudaStream_t s) {
    dim3 blk(32, 4);
    dim3 grd((G.nr + G.g + blk.x - 1) / blk.x, (G.nz + G.g + blk.y - 1) / blk.y);
    add_kernel<<<grd, blk, 0, s>>>(G, out, c, x);
}

int wave_stage_blocks(const LevelGeom& G) {
    const int nx = (G.nr + G.g + kWaveBX - 1) / kWaveBX, ny = (G.nz + G.g + kWaveBY - 1) / kWaveBY;
    return nx * ny;
}

void launch_wave_stage(const WaveArgs& a, cudaStream_t s) {
    dim3 blk(kWaveBX, kWaveBY);
    dim3 grd((a.G.nr + a.G.g + kWaveBX - 1) / kWaveBX, (a.G.nz + a.G.g + kWaveBY - 1) / kWaveBY);
    if (a.physical) wave_stage_kernel<true><<<grd, blk, 0, s>>>(a);
    else wave_stage_kernel<false><<<grd, blk, 0, s>>>(a);
}

int max_coeff_blocks(const LevelGeom& G) {
    const int nx = (G.nr + G.g + kMaxBX - 1) / kMaxBX, ny = (G.nz + G.g + kMaxBY - 1) / kMaxBY;
    return nx * ny;
}

void launch_max_coeffs(const MaxCoeffArgs& a, cudaStream_t s) {
    dim3 blk(kMaxBX, kMaxBY);
    dim3 grd((a.G.nr + a.G.g + kMaxBX - 1) / kMaxBX, (a.G.nz + a.G.g + kMaxBY - 1) / kMaxBY);
    max_coeff_kernel<<<grd, blk, 0, s>>>(a);
}

void launch_sor_coeffs(const SorCoeffArgs& a, cudaStream_t s) {
    dim3 blk(32, 4);
    dim3 grd((a.G.nr + a.G.g + blk.x - 1) / blk.x, (a.G.nz + a.G.g + blk.y - 1) / blk.y);
    sor_coeff_kernel<<<grd, blk, 0, s>>>(a);
}

void launch_sor_phys_pass(const SorPhysPassArgs& a, cudaStream_t s) {
    const int ni = a.G.nr + a.G.g - 2, nj = (a.G.nz + a.G.g - 2 + 1) / 2;
    dim3 blk(kSorBX, kSorBY);
    dim3 grd((ni + kSorBX - 1) / kSorBX, (nj + kSorBY - 1) / kSorBY);
    sor_phys_pass_kernel<<<grd, blk, 0, s>>>(a);
}

void launch_sor_phys_pass_seq(const SorPhysPassArgs& a, cudaStream_t s) {
    sor_phys_pass_seq_kernel<<<1, kSeqThreads, 0, s>>>(a);
}

void launch_wave_residual(const double* partial, int nparts, int nr, int nz, EllCtl* ctl, cudaStream_t s) {
    wave_residual_kernel<<<1, 256, 0, s>>>(partial, nparts, nr, nz, ctl);
}

void launch_pulse_xi(const PulseCoeffArgs& a, cudaStream_t s) {
    dim3 blk(32, 4);
    const int ni = a.G.axis ? a.G.nr : a.G.nr + a.G.g;
    dim3 grd((ni + blk.x - 1) / blk.x, (a.G.nz - a.G.jlo + 1 + blk.y - 1) / blk.y);
    pulse_xi_kernel<<<grd, blk, 0, s>>>(a);
}

void launch_pulse_coeffs(const PulseCoeffArgs& a, cudaStream_t s) {
    dim3 blk(32, 4);
    dim3 grd((a.G.nr + a.G.g + blk.x - 1) / blk.x, (a.G.nz + a.G.g + blk.y - 1) / blk.y);
    pulse_coeff_kernel<<<grd, blk, 0, s>>>(a);
}

}  // namespace ollin
