// synth.cu -- seeded synthetic initial states (device).
//
// Entropy bump: s1 = 1e-4 * c_p * exp(-|x-x_c|^2 / (2 sigma^2)), c_p = 2.5 R_gas.
// Dipole: B_r = 2 B0 (r_b/r)^3 cos(theta), B_theta = B0 (r_b/r)^3 sin(theta) in
// the Yin frame, B0 = 1e-3 sqrt(rho_b) c_s(r_b); Yang blocks get the field
// rotated into their frame like ModInitiation_B_uniform_Bph does
// (3_6/ModInitiation.f90:143-188).
// Velocity (kind 1): 512 Fourier modes, |k| log-uniform in
// [2 pi / shell thickness, 2 pi / (8 dr)], amplitude |k|^(-1/3) (so the band
// energy follows k^(-5/3)), random direction, solenoidal polarisation and
// phase; evaluated in global Cartesian coordinates at interior cell centres
// (ghosts are filled by the exchange, as ModInitiation_rand_velocity leaves
// them to it), converted to the block's frame, then scaled to rms Mach `mach`
// against the local c_s(r).
#include "synth.cuh"

#include <cmath>
#include <random>
#include <vector>

namespace falcon {

namespace {

constexpr int NMODE = 512;

struct Mode { float kx, ky, kz, ex, ey, ez, amp, phase; };

struct SynthParams {
    double xc[3], sig, s_amp, B0, rb;
    int nmode;
    int with_v;
};

__device__ __forceinline__ void yy_conv_d(double r, double t, double p, double& t2, double& p2) {
    const double st = sin(t), ct = cos(t), sp = sin(p), cp = cos(p);
    t2 = acos(st * sp);
    p2 = copysign(fabs(acos(-(st * cp) / sqrt(st * st * (cp * cp) + ct * ct))), ct);
}

// rotate the (theta, phi) components of a vector given at frame point (t,p)
// into the other panel's frame (3_6/ModYinYang.f90:34-46)
__device__ __forceinline__ void yy_vec_d(double t, double p, double& v2, double& v3) {
    double t2, p2;
    yy_conv_d(1.0, t, p, t2, p2);
    const double a = sin(p) * sin(p2), c = cos(p) / sin(t2);
    const double o2 = -(a * v2) - c * v3;
    const double o3 = -(a * v3) + c * v2;
    v2 = o2; v3 = o3;
}

template <class T>
__global__ void k_synth(T* U, const double* xj, const double* xk, Geometry geo, StepDims d, SynthParams sp,
                        const Mode* modes, double* sumsq) {
    const int b = blockIdx.y;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    double local = 0.0;
    if (q < d.ncell) {
        const int ip = q % d.nip, jp = (q / d.nip) % d.njp, kp = q / (d.nip * d.njp);
        const bool yin = geo.flags[b] & 1;
        const double r = geo.gi[(size_t)b * GI_COUNT * d.nip + GI_R * d.nip + ip];
        const double t = xj[(size_t)b * d.njp + jp], p = xk[(size_t)b * d.nkp + kp];
        double ty = t, py = p;
        if (!yin) yy_conv_d(r, t, p, ty, py);
        const double x = r * sin(ty) * cos(py), y = r * sin(ty) * sin(py), z = r * cos(ty);
        const double dx = x - sp.xc[0], dy = y - sp.xc[1], dz = z - sp.xc[2];
        const double s1 = sp.s_amp * exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * sp.sig * sp.sig));
        const double qq = (sp.rb / r) * (sp.rb / r) * (sp.rb / r);
        double br = 2.0 * sp.B0 * qq * cos(ty), bt = sp.B0 * qq * sin(ty), bp = 0.0;
        if (!yin) yy_vec_d(ty, py, bt, bp);
        T* c = U + (size_t)b * NV * d.ncell + q;
        const size_t n = d.ncell;
        c[V_RHO1 * n] = T(0);
        c[V_S1 * n] = (T)s1;
        c[V_BR * n] = (T)br;
        c[V_BT * n] = (T)bt;
        c[V_BP * n] = (T)bp;
        double vr = 0, vt = 0, vp = 0;
        const bool interior = ip >= 2 && ip < d.nip - 2 && jp >= 2 && jp < d.njp - 2 && kp >= 2 && kp < d.nkp - 2;
        if (sp.with_v && interior) {
            float vx = 0.f, vy = 0.f, vz = 0.f;
            const float fx = (float)x, fy = (float)y, fz = (float)z;
            for (int m = 0; m < sp.nmode; ++m) {
                const Mode M = modes[m];
                const float ph = M.kx * fx + M.ky * fy + M.kz * fz + M.phase;
                const float a = M.amp * cosf(ph);
                vx += a * M.ex; vy += a * M.ey; vz += a * M.ez;
            }
            const double st = sin(ty), ct = cos(ty), sph = sin(py), cph = cos(py);
            vr = st * cph * vx + st * sph * vy + ct * vz;
            vt = ct * cph * vx + ct * sph * vy - st * vz;
            vp = -sph * vx + cph * vy;
            if (!yin) yy_vec_d(ty, py, vt, vp);
            local = vr * vr + vt * vt + vp * vp;
        }
        c[V_VR * n] = (T)vr;
        c[V_VT * n] = (T)vt;
        c[V_VP * n] = (T)vp;
    }
    // the CTA's sum of |v|^2 into its own slot (summed on the host in a fixed
    // order, so the scale and the seeded state are the same on every run)
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    __shared__ double ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += ws[w];
        sumsq[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
    }
}

template <class T>
__global__ void k_scale_v(T* U, Geometry geo, StepDims d, double scale) {
    const int b = blockIdx.y;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.ncell) return;
    const int ip = q % d.nip;
    const double* Gi = geo.gi + (size_t)b * GI_COUNT * d.nip;
    // local sound speed c_s = sqrt(gamma1 p0/rho0) = Xi * CS column
    const double A1 = Gi[GI_A1 * d.nip + ip];   // gamma1*p0/rho0
    const double f = scale * sqrt(A1);
    T* c = U + (size_t)b * NV * d.ncell + q;
    const size_t n = d.ncell;
    c[V_VR * n] = (T)((double)c[V_VR * n] * f);
    c[V_VT * n] = (T)((double)c[V_VT * n] * f);
    c[V_VP * n] = (T)((double)c[V_VP * n] * f);
}

}  // namespace

std::string synth_initial_state(const Grid& g, const Geometry& geo, void* U, bool mixed, int kind, uint64_t seed,
                                double mach, cudaStream_t st) {
    std::mt19937_64 rng(seed);
    auto uni = [&](double a, double b) { return a + (b - a) * ((double)(rng() >> 11) * (1.0 / 9007199254740992.0)); };
    const double kRsun = (double)6.955e10f;
    const double pi = 3.14159265358979323846;
    SynthParams sp{};
    const double rc = uni(0.75, 0.95) * kRsun, tc = uni(pi / 3, 2 * pi / 3), pc = uni(-pi / 2, pi / 2);
    sp.sig = uni(0.03, 0.08) * kRsun;
    sp.xc[0] = rc * std::sin(tc) * std::cos(pc);
    sp.xc[1] = rc * std::sin(tc) * std::sin(pc);
    sp.xc[2] = rc * std::cos(tc);
    sp.s_amp = 1e-4 * 2.5 * g.bg.R_gas;
    sp.rb = g.r_range[0];
    sp.B0 = 1e-3 * std::sqrt(g.bg.rho_b) * std::sqrt((double)(5.0f / 3.0f) * g.bg.p_b / g.bg.rho_b);
    sp.with_v = kind == 1;
    sp.nmode = NMODE;
    std::vector<Mode> modes(NMODE);
    double dr_min = 1e300;
    for (int b = 0; b < g.nblocks; ++b) dr_min = std::min(dr_min, g.dx[3 * b]);
    const double kmin = 2 * pi / (g.r_range[1] - g.r_range[0]), kmax = 2 * pi / (8 * dr_min);
    for (auto& M : modes) {
        const double kk = std::exp(uni(std::log(kmin), std::log(kmax)));
        const double ct = uni(-1, 1), ph = uni(0, 2 * pi), st_ = std::sqrt(1 - ct * ct);
        const double kx = st_ * std::cos(ph), ky = st_ * std::sin(ph), kz = ct;
        // orthonormal basis perpendicular to k
        double ax = std::fabs(kz) < 0.9 ? 0 : 1, ay = 0, az = std::fabs(kz) < 0.9 ? 1 : 0;
        double e1x = ay * kz - az * ky, e1y = az * kx - ax * kz, e1z = ax * ky - ay * kx;
        const double n1 = std::sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
        e1x /= n1; e1y /= n1; e1z /= n1;
        const double e2x = ky * e1z - kz * e1y, e2y = kz * e1x - kx * e1z, e2z = kx * e1y - ky * e1x;
        const double al = uni(0, 2 * pi);
        M.kx = (float)(kk * kx); M.ky = (float)(kk * ky); M.kz = (float)(kk * kz);
        M.ex = (float)(std::cos(al) * e1x + std::sin(al) * e2x);
        M.ey = (float)(std::cos(al) * e1y + std::sin(al) * e2y);
        M.ez = (float)(std::cos(al) * e1z + std::sin(al) * e2z);
        M.amp = (float)std::pow(kk / kmin, -1.0 / 3.0);
        M.phase = (float)uni(0, 2 * pi);
    }
    StepDims d{g.nblocks, g.ni, g.nj, g.nk, g.nip, g.njp, g.nkp, g.ncell};
    double *dxj = nullptr, *dxk = nullptr, *dsum = nullptr;
    Mode* dmodes = nullptr;
    auto cleanup = [&] { cudaFree(dxj); cudaFree(dxk); cudaFree(dsum); cudaFree(dmodes); };
    cudaError_t e = cudaMalloc(&dxj, g.xj.size() * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dxk, g.xk.size() * 8);
    dim3 grid((g.ncell + 255) / 256, g.nblocks);
    const size_t nslot = (size_t)grid.x * grid.y;   // one partial sum per CTA
    if (e == cudaSuccess) e = cudaMalloc(&dsum, nslot * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dmodes, sizeof(Mode) * NMODE);
    if (e == cudaSuccess) e = cudaMemcpy(dxj, g.xj.data(), g.xj.size() * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dxk, g.xk.data(), g.xk.size() * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dmodes, modes.data(), sizeof(Mode) * NMODE, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cleanup(); return std::string("synth setup: ") + cudaGetErrorString(e); }
    if (mixed) k_synth<float><<<grid, 256, 0, st>>>((float*)U, dxj, dxk, geo, d, sp, dmodes, dsum);
    else k_synth<double><<<grid, 256, 0, st>>>((double*)U, dxj, dxk, geo, d, sp, dmodes, dsum);
    double sumsq = 0;
    std::vector<double> part(nslot);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), dsum, nslot * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (double x : part) sumsq += x;
    if (e == cudaSuccess && kind == 1 && sumsq > 0) {
        const double nint = (double)g.nblocks * g.ni * g.nj * g.nk;
        const double vrms = std::sqrt(sumsq / nint);
        const double scale = mach / vrms;
        if (mixed) k_scale_v<float><<<grid, 256, 0, st>>>((float*)U, geo, d, scale);
        else k_scale_v<double><<<grid, 256, 0, st>>>((double*)U, geo, d, scale);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cleanup();
    if (e != cudaSuccess) return std::string("synth: ") + cudaGetErrorString(e);
    return "";
}

}  // namespace falcon
