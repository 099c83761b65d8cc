// output.cu -- device side of the AllCells plot output (ModSave_AllCells,
// 3_6/ModSavePlot.f90:520-650): per block, the (ni+1)(nj+1)(nk+1) cell
// corners with the average of the 8 surrounding cell centres, position and
// the vectors in Cartesian components. Compiled with -fmad=false so that the
// FP64 path reproduces the reference's arithmetic bit for bit; the file
// text is written on the host (capi.cu).
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace falcon {
namespace {

// value of variable v at padded cell `c` of block b, as the host download
// gives it (the mixed path adds the 8-bit correction of u^n)
template <class T>
__device__ __forceinline__ double cell_value(const T* U, const int8_t* lo, const T* psi, int64_t b, int v, int64_t c,
                                             const StepDims& d) {
    const int64_t ncell = d.ncell;
    if (v == NV) return psi ? (double)psi[b * ncell + c] : 0.0;
    const int64_t e = (b * NV + v) * ncell + c;
    const T hi = U[e];
    double x = (double)hi;
    if constexpr (sizeof(T) == 4) {
        const int64_t q = lo ? lo_index(e, d) : -1;
        if (q >= 0) x += (double)lo[q] * (double)lo_unit((float)hi);
    }
    return x;
}

template <class T>
__global__ void __launch_bounds__(256) k_allcells(const T* U, const int8_t* lo, const T* psi, const double* tab,
                                                  int b0, int nbb, StepDims d, double* out) {
    const int nci = d.ni + 1, ncj = d.nj + 1, nck = d.nk + 1;
    const int64_t ncor = (int64_t)nci * ncj * nck;
    const int tstride = allcells_table_stride(d);
    const double rsun = (double)6.955e10f;   // R_sun__CGS, a default-real constant (3_6/ModConst.f90:5)
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < (int64_t)nbb * ncor;
         x += (int64_t)gridDim.x * blockDim.x) {
        const int64_t bb = x / ncor, cq = x - bb * ncor;
        const int i = (int)(cq % nci), j = (int)((cq / nci) % ncj), k = (int)(cq / ((int64_t)nci * ncj));
        const int64_t b = b0 + bb;
        // Fortran corner (i+1, j+1, k+1) averages cells (i..i+1, j..j+1, k..k+1);
        // Fortran cell index m sits at padded index m + 1 (two ghost layers)
        auto cell = [&](int fi, int fj, int fk) -> int64_t {
            return (int64_t)(fi + 1) + (int64_t)d.nip * ((fj + 1) + (int64_t)d.njp * (fk + 1));
        };
        double val[NV + 1];
#pragma unroll
        for (int v = 0; v <= NV; ++v) {
            auto f = [&](int di, int dj, int dk) { return cell_value(U, lo, psi, b, v, cell(i + di, j + dj, k + dk), d); };
            // 0.125d0*(8 neighbours), summed left to right (3_6/ModSavePlot.f90:575-580)
            double s = f(0, 0, 0) + f(1, 0, 0);
            s = s + f(0, 1, 0);
            s = s + f(1, 1, 0);
            s = s + f(0, 0, 1);
            s = s + f(1, 0, 1);
            s = s + f(0, 1, 1);
            s = s + f(1, 1, 1);
            val[v] = 0.125 * s;
        }
        const double* t = tab + b * tstride;
        const double r = t[i], sth = t[nci + j], cth = t[nci + ncj + j];
        const double sph = t[nci + 2 * ncj + k], cph = t[nci + 2 * ncj + nck + k];
        const bool yin = t[nci + 2 * ncj + 2 * nck] != 0.0;
        double* o = out + x * 12;
        // position in units of R_sun; Yang: (x, y, z) = (-x0, z0, y0)
        if (yin) {
            o[0] = r * sth * cph;
            o[1] = r * sth * sph;
            o[2] = r * cth;
        } else {
            o[0] = -(r * sth * cph);
            o[1] = r * cth;
            o[2] = r * sth * sph;
        }
        o[0] = o[0] / rsun;
        o[1] = o[1] / rsun;
        o[2] = o[2] / rsun;
        // (vr, vt, vp) and (br, bt, bp) -> Cartesian, the same Yang mapping
        auto cart = [&](int a) {
            const double vx = val[a] * sth * cph + val[a + 1] * cth * cph - val[a + 2] * sph;
            const double vy = val[a] * sth * sph + val[a + 1] * cth * sph + val[a + 2] * cph;
            const double vz = val[a] * cth - val[a + 1] * sth;
            if (yin) { val[a] = vx; val[a + 1] = vy; val[a + 2] = vz; }
            else { val[a] = -vx; val[a + 1] = vz; val[a + 2] = vy; }
        };
        cart(V_VR);
        cart(V_BR);
#pragma unroll
        for (int v = 0; v <= NV; ++v) o[3 + v] = val[v];
    }
}

}  // namespace

cudaError_t launch_allcells(const StepDims& d, const void* U, const int8_t* lo, const void* psi, bool fp32,
                            const double* tab, int b0, int nbb, double* out, cudaStream_t st) {
    if (fp32)
        k_allcells<float><<<1216, 256, 0, st>>>((const float*)U, lo, (const float*)psi, tab, b0, nbb, d, out);
    else
        k_allcells<double><<<1216, 256, 0, st>>>((const double*)U, nullptr, (const double*)psi, tab, b0, nbb, d, out);
    return cudaGetLastError();
}

}  // namespace falcon
