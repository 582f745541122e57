// readouts.cu — per-element strain and stress of a configuration (core/fields.py), on the
// device: one thread per triangle, FP64.
//
//   F = Ds B                                   (Ds: edge vectors as columns, B = Dm^-1)
//   E = (F^T F - I) / 2,  E_zz = 0             Green-Lagrange strain (plane strain)
//   sigma = (mu F F^T + (lam ln J - mu) I) / J, sigma_zz = lam ln J / J   (Neo-Hookean Cauchy)
//   von Mises: strain sqrt(2/3 e':e'), stress sqrt(3/2 s':s')  (' deviatoric, 3 x 3)
//   signed: the in-plane principal value of larger magnitude, with its sign
#include <cuda_runtime.h>
#include <stdint.h>

#include "d2f_solver.h"

namespace {

// deviatoric squared norm of the 3 x 3 tensor [[a, b, 0], [b, d, 0], [0, 0, z]]
__device__ __forceinline__ double dev_norm2(double a, double b, double d, double z) {
    const double m = (a + d + z) / 3.0;
    const double da = a - m, dd = d - m, dz = z - m;
    return da * da + dd * dd + dz * dz + 2.0 * b * b;
}

// in-plane principal value of larger magnitude of [[a, b], [b, d]]
__device__ __forceinline__ double signed_principal(double a, double b, double d) {
    const double m = 0.5 * (a + d), r = sqrt(0.25 * (a - d) * (a - d) + b * b);
    const double hi = m + r, lo = m - r;
    return fabs(hi) >= fabs(lo) ? hi : lo;
}

__global__ void element_fields_kernel(int T, const int32_t *__restrict__ tri, const double *__restrict__ Bm,
                                      const double *__restrict__ mu, const double *__restrict__ lam,
                                      const double *__restrict__ x, double *strain_vm, double *strain_signed,
                                      double *stress_vm, double *stress_signed) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
        const int i0 = tri[3 * t], i1 = tri[3 * t + 1], i2 = tri[3 * t + 2];
        const double e1x = x[2 * i1] - x[2 * i0], e1y = x[2 * i1 + 1] - x[2 * i0 + 1];
        const double e2x = x[2 * i2] - x[2 * i0], e2y = x[2 * i2 + 1] - x[2 * i0 + 1];
        const double b00 = Bm[4 * t], b01 = Bm[4 * t + 1], b10 = Bm[4 * t + 2], b11 = Bm[4 * t + 3];
        const double F00 = e1x * b00 + e2x * b10, F01 = e1x * b01 + e2x * b11;
        const double F10 = e1y * b00 + e2y * b10, F11 = e1y * b01 + e2y * b11;
        // Green-Lagrange strain
        const double E00 = 0.5 * (F00 * F00 + F10 * F10 - 1.0), E11 = 0.5 * (F01 * F01 + F11 * F11 - 1.0);
        const double E01 = 0.5 * (F00 * F01 + F10 * F11);
        if (strain_vm) strain_vm[t] = sqrt(2.0 / 3.0 * dev_norm2(E00, E01, E11, 0.0));
        if (strain_signed) strain_signed[t] = signed_principal(E00, E01, E11);
        if (stress_vm || stress_signed) {
            const double J = F00 * F11 - F01 * F10;
            const double lnJ = log(J > 1.0e-12 ? J : 1.0e-12);
            const double m = mu[t], l = lam[t], c = l * lnJ - m;
            const double S00 = (m * (F00 * F00 + F01 * F01) + c) / J, S11 = (m * (F10 * F10 + F11 * F11) + c) / J;
            const double S01 = m * (F00 * F10 + F01 * F11) / J, Szz = l * lnJ / J;
            if (stress_vm) stress_vm[t] = sqrt(1.5 * dev_norm2(S00, S01, S11, Szz));
            if (stress_signed) stress_signed[t] = signed_principal(S00, S01, S11);
        }
    }
}

}  // namespace

extern "C" int32_t d2f_element_fields(int32_t T, const int32_t *tri, const double *Bm, const double *mu,
                                      const double *lam, const double *x, double *strain_vm,
                                      double *strain_signed, double *stress_vm, double *stress_signed,
                                      void *stream) {
    g_err[0] = 0;
    if (T <= 0 || !tri || !Bm || !x) return d2f_fail(D2F_EINVAL, "d2f_element_fields: empty mesh or null input");
    if ((stress_vm || stress_signed) && (!mu || !lam))
        return d2f_fail(D2F_EINVAL, "d2f_element_fields: stress needs mu and lam");
    const int threads = 256;
    int blocks = (T + threads - 1) / threads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    element_fields_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(T, tri, Bm, mu, lam, x, strain_vm, strain_signed,
                                                                       stress_vm, stress_signed);
    if (cudaGetLastError() != cudaSuccess) return d2f_fail(D2F_ECUDA, "d2f_element_fields: launch failed");
    return D2F_OK;
}
