// qr_coef.cu -- coefficient updates on the device (qr_op_set_coeffs_device).
//
// The plan tables of qr_apply depend on the coefficients only through sums of
// the merged coefficients c_m with signs; which strings, in which order and
// with which signs is fixed when the plan is built (host).  These kernels
// redo exactly those FP64 operations from a new coefficient vector on the
// device, so a training loop that changes c every step never waits for the
// host, and the tables come out bit-identical to a fresh host build.
//   1. merge_coeffs_kernel: c'_k = m(phase_k) * c_k (make_params,
//      qrusty/src/accel.rs:141-157, num-complex product), folded per merged
//      (x, z) string in input order (first term, then additions);
//   2. coef_program_kernel: every table entry / coefficient of a plan
//      (CoefSlot), as the host plan builder forms it.
#include "qr_common.cuh"

namespace qr {

__global__ void __launch_bounds__(256) merge_coeffs_kernel(uint32_t M, const uint32_t *mm_off,
                                                           const uint32_t *mm_terms,
                                                           const double2 *coeff,
                                                           const uint8_t *phase, double2 *mc) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        double2 v = make_double2(0.0, 0.0);
        for (uint32_t t = mm_off[i]; t < mm_off[i + 1]; ++t) {
            const uint32_t k = mm_terms[t];
            const double2 c = make_param(coeff[k], phase[k]);
            if (t == mm_off[i]) {
                v = c;
            } else {
                v.x = __dadd_rn(v.x, c.x);
                v.y = __dadd_rn(v.y, c.y);
            }
        }
        mc[i] = v;
    }
}

__device__ __forceinline__ double2 plan_coef(const double2 *mc, const uint8_t *madj, uint32_t m,
                                             int adjoint) {
    double2 c = mc[m];
    if (adjoint) {
        c.y = -c.y;
        if (madj[m]) {
            c.x = -c.x;
            c.y = -c.y;
        }
    }
    return c;
}

__global__ void __launch_bounds__(256) coef_program_kernel(const CoefSlot *slots, uint32_t nslots,
                                                           const uint32_t *mem,
                                                           const uint8_t *coord,
                                                           const double2 *mc, const uint8_t *madj,
                                                           int adjoint) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nslots;
         i += gridDim.x * blockDim.x) {
        const CoefSlot S = slots[i];
        if (S.kind == 2) {
            *reinterpret_cast<double2 *>(S.dst) = plan_coef(mc, madj, mem[S.m0], adjoint);
            continue;
        }
        const uint32_t ent = 1u << S.d;
        for (uint32_t u = 0; u < ent; ++u) {
            double ar = 0.0, ai = 0.0;
            for (uint32_t kk = S.m0; kk < S.m0 + S.cnt; ++kk) {
                const double2 c = plan_coef(mc, madj, mem[kk], adjoint);
                if (__popc(u & coord[kk]) & 1) {
                    ar = __dsub_rn(ar, c.x);
                    ai = __dsub_rn(ai, c.y);
                } else {
                    ar = __dadd_rn(ar, c.x);
                    ai = __dadd_rn(ai, c.y);
                }
            }
            if (S.kind == 0)
                reinterpret_cast<float2 *>(S.dst)[u] =
                    make_float2(__double2float_rn(ar), __double2float_rn(ai));
            else
                reinterpret_cast<double2 *>(S.dst)[u] = make_double2(ar, ai);
        }
    }
}

static unsigned grid_for(uint32_t n) {
    const uint32_t g = (n + 255u) / 256u;
    return g == 0 ? 1u : (g > 4096u ? 4096u : g);
}

cudaError_t launch_merge_coeffs(uint32_t M, const uint32_t *mm_off, const uint32_t *mm_terms,
                                const double2 *coeff, const uint8_t *phase, double2 *mc,
                                cudaStream_t st) {
    if (M == 0) return cudaSuccess;
    merge_coeffs_kernel<<<grid_for(M), 256, 0, st>>>(M, mm_off, mm_terms, coeff, phase, mc);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_coef_program(const CoefSlot *slots, uint32_t nslots, const uint32_t *mem,
                                const uint8_t *coord, const double2 *mc, const uint8_t *madj,
                                int adjoint, cudaStream_t st) {
    if (nslots == 0) return cudaSuccess;
    coef_program_kernel<<<grid_for(nslots), 256, 0, st>>>(slots, nslots, mem, coord, mc, madj,
                                                          adjoint);
    count_launch();
    return cudaGetLastError();
}

}  // namespace qr
