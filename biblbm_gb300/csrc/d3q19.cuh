// D3Q19 lattice constants and the per-cell collision arithmetic shared by the
// lattice and immersed-boundary kernels.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "bib_internal.h"

namespace bib {

// Velocity set in the reference order, src/latticeBoltzmann/nearestNeighborLattices3D.hh:165-197
// (c[i] = -c[i+9]).
__host__ __device__ constexpr int cx(int i) {
    return (i == 1 || i == 4 || i == 5 || i == 6 || i == 7) ? -1 : ((i == 10 || i == 13 || i == 14 || i == 15 || i == 16) ? 1 : 0);
}
__host__ __device__ constexpr int cy(int i) {
    return (i == 2 || i == 4 || i == 8 || i == 9 || i == 14) ? -1 : ((i == 5 || i == 11 || i == 13 || i == 17 || i == 18) ? 1 : 0);
}
__host__ __device__ constexpr int cz(int i) {
    return (i == 3 || i == 6 || i == 8 || i == 16 || i == 18) ? -1 : ((i == 7 || i == 9 || i == 12 || i == 15 || i == 17) ? 1 : 0);
}
__host__ __device__ constexpr int opposite(int i) { return i == 0 ? 0 : (i < 10 ? i + 9 : i - 9); }

template <class C>
__host__ __device__ constexpr C weight(int i) {
    return i == 0 ? C(1) / C(3) : ((cx(i) * cx(i) + cy(i) * cy(i) + cz(i) * cz(i)) == 1 ? C(1) / C(18) : C(1) / C(36));
}

// ---------------------------------------------------------------- storage
// Populations are stored as f-bar = f - t_i; FP16 storage keeps f-bar * scale.
template <class T>
struct Store;
template <>
struct Store<double> {
    using C = double;
    using F = double;
    using U = double;  // velocity field
    static __device__ __forceinline__ double load(const double* p, float) { return __ldg(p); }
    static __device__ __forceinline__ void store(double* p, double v, float) { *p = v; }
};
template <>
struct Store<float> {
    using C = float;
    using F = float;
    using U = float;
    static __device__ __forceinline__ float load(const float* p, float) { return __ldg(p); }
    static __device__ __forceinline__ void store(float* p, float v, float) { *p = v; }
};
template <>
struct Store<__half> {
    using C = float;
    using F = float;
    using U = __half;  // the velocity field in FP16 too: it only feeds the interpolation
    static __device__ __forceinline__ float load(const __half* p, float inv_scale) {
        return __half2float(__ldg(p)) * inv_scale;
    }
    static __device__ __forceinline__ void store(__half* p, float v, float scale) { *p = __float2half_rn(v * scale); }
};

// ---------------------------------------------------------------- moments
// get_rhoBar and get_rhoBar_j (partial sums), src/latticeBoltzmann/momentTemplates3D.h:350-423
template <class C>
__device__ __forceinline__ C rho_bar_seq(const C* f) {
    return f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14] +
           f[15] + f[16] + f[17] + f[18];
}
template <class C>
__device__ __forceinline__ void rho_bar_j(const C* f, C& rb, C* j) {
    const C sxm = f[1] + f[4] + f[5] + f[6] + f[7];
    const C sxp = f[10] + f[13] + f[14] + f[15] + f[16];
    const C sym = f[2] + f[4] + f[8] + f[9] + f[14];
    const C syp = f[5] + f[11] + f[13] + f[17] + f[18];
    const C szm = f[3] + f[6] + f[8] + f[16] + f[18];
    const C szp = f[7] + f[9] + f[12] + f[15] + f[17];
    const C sx0 = f[0] + f[2] + f[3] + f[8] + f[9] + f[11] + f[12] + f[17] + f[18];
    rb = sxm + sx0 + sxp;
    j[0] = sxp - sxm;
    j[1] = syp - sym;
    j[2] = szp - szm;
}
// ExternalForceDynamics::computeVelocity, src/basicDynamics/externalForceDynamics.hh:59-74
template <class C>
__device__ __forceinline__ void velocity_with_force(const C* f, const C* F, C* u) {
    C rb, j[3];
    rho_bar_j(f, rb, j);
    const C inv = C(1) / (rb + C(1));
    u[0] = j[0] * inv + F[0] / C(2);
    u[1] = j[1] * inv + F[1] / C(2);
    u[2] = j[2] * inv + F[2] / C(2);
}

// bgk_ma2_equilibrium, src/latticeBoltzmann/dynamicsTemplates3D.h:675-678
template <class C>
__device__ __forceinline__ C bgk_equilibrium(int i, C rhoBar, C invRho, const C* j, C jSqr) {
    const C c_j = C(cx(i)) * j[0] + C(cy(i)) * j[1] + C(cz(i)) * j[2];
    return weight<C>(i) * (rhoBar + C(3) * c_j + invRho * (C(4.5) * c_j * c_j - C(1.5) * jSqr));
}

// bgk_ma2_collision_base, src/latticeBoltzmann/dynamicsTemplates3D.h:770-838
template <class C>
__device__ __forceinline__ void bgk_collision(C* f, C rhoBar, const C* j, C omega, C invRho) {
    const C omo = C(1) - omega;
    const C t0w = weight<C>(0) * omega, t1w = weight<C>(1) * omega, t4w = weight<C>(4) * omega;
    const C jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    const C kx = C(3) * j[0], ky = C(3) * j[1], kz = C(3) * j[2];
    const C kxS = invRho / C(2) * kx * kx, kyS = invRho / C(2) * ky * ky, kzS = invRho / C(2) * kz * kz;
    const C kxky = invRho * kx * ky, kxkz = invRho * kx * kz, kykz = invRho * ky * kz;
    const C C1 = rhoBar + invRho * C(3) * jSqr;
    C C2, C3;
    C3 = -kxS - kyS - kzS;
    f[0] = f[0] * omo + t0w * (C1 + C3);
#define BIB_PAIR(a, b, tw)                      \
    f[a] = f[a] * omo + tw * (C1 + C2 + C3); \
    f[b] = f[b] * omo + tw * (C1 - C2 + C3);
    C2 = -kx; C3 = -kyS - kzS; BIB_PAIR(1, 10, t1w)
    C2 = -ky; C3 = -kxS - kzS; BIB_PAIR(2, 11, t1w)
    C2 = -kz; C3 = -kxS - kyS; BIB_PAIR(3, 12, t1w)
    C2 = -kx - ky; C3 = kxky - kzS; BIB_PAIR(4, 13, t4w)
    C2 = -kx + ky; C3 = -kxky - kzS; BIB_PAIR(5, 14, t4w)
    C2 = -kx - kz; C3 = kxkz - kyS; BIB_PAIR(6, 15, t4w)
    C2 = -kx + kz; C3 = -kxkz - kyS; BIB_PAIR(7, 16, t4w)
    C2 = -ky - kz; C3 = kykz - kxS; BIB_PAIR(8, 17, t4w)
    C2 = -ky + kz; C3 = -kykz - kxS; BIB_PAIR(9, 18, t4w)
#undef BIB_PAIR
}

// Guo forcing for D3Q19, src/fsi/VariableViscosityDynamics.hh:47-129
template <class C>
__device__ __forceinline__ void guo_force(C* f, const C* F, const C* u, C omega) {
    const C mu = C(1) - omega / C(2);
    const C o6 = C(1) / C(6), o12 = C(1) / C(12);
    const C F0 = F[0], F1 = F[1], F2 = F[2], u0 = u[0], u1 = u[1], u2 = u[2];
    f[0] += -mu * (F0 * u0 + F1 * u1 + F2 * u2);
    f[1] += o6 * mu * (F0 * (C(-1) + 2 * u0) - F1 * u1 - F2 * u2);
    f[2] += -o6 * mu * (F0 * u0 + F1 * (C(1) - 2 * u1) + F2 * u2);
    f[3] += -o6 * mu * (F0 * u0 + F1 * u1 + F2 * (C(1) - 2 * u2));
    f[4] += o12 * mu * (F0 * (C(-1) + 2 * u0 + 3 * u1) + F1 * (C(-1) + 2 * u1 + 3 * u0) - F2 * u2);
    f[5] += o12 * mu * (F0 * (C(-1) + 2 * u0 - 3 * u1) + F1 * (C(1) + 2 * u1 - 3 * u0) - F2 * u2);
    f[6] += o12 * mu * (F0 * (C(-1) + 2 * u0 + 3 * u2) - F1 * u1 + F2 * (C(-1) + 2 * u2 + 3 * u0));
    f[7] += o12 * mu * (F0 * (C(-1) + 2 * u0 - 3 * u2) - F1 * u1 + F2 * (C(1) + 2 * u2 - 3 * u0));
    f[8] += -o12 * mu * (F0 * u0 + F1 * (C(1) - 2 * u1 - 3 * u2) + F2 * (C(1) - 2 * u2 - 3 * u1));
    f[9] += -o12 * mu * (F0 * u0 + F1 * (C(1) - 2 * u1 + 3 * u2) + F2 * (C(-1) - 2 * u2 + 3 * u1));
    f[10] += o6 * mu * (F0 * (C(1) + 2 * u0) - F1 * u1 - F2 * u2);
    f[11] += -o6 * mu * (F0 * u0 + F1 * (C(-1) - 2 * u1) + F2 * u2);
    f[12] += -o6 * mu * (F0 * u0 + F1 * u1 + F2 * (C(-1) - 2 * u2));
    f[13] += o12 * mu * (F0 * (C(1) + 2 * u0 + 3 * u1) + F1 * (C(1) + 2 * u1 + 3 * u0) - F2 * u2);
    f[14] += o12 * mu * (F0 * (C(1) + 2 * u0 - 3 * u1) + F1 * (C(-1) + 2 * u1 - 3 * u0) - F2 * u2);
    f[15] += o12 * mu * (F0 * (C(1) + 2 * u0 + 3 * u2) - F1 * u1 + F2 * (C(1) + 2 * u2 + 3 * u0));
    f[16] += o12 * mu * (F0 * (C(1) + 2 * u0 - 3 * u2) - F1 * u1 + F2 * (C(-1) + 2 * u2 - 3 * u0));
    f[17] += -o12 * mu * (F0 * u0 + F1 * (C(-1) - 2 * u1 - 3 * u2) + F2 * (C(-1) - 2 * u2 - 3 * u1));
    f[18] += -o12 * mu * (F0 * u0 + F1 * (C(-1) - 2 * u1 + 3 * u2) + F2 * (C(1) - 2 * u2 + 3 * u1));
}

// Collision of one cell.  BGK_GUO_VOF follows GuoExternalForceVOFDynamics::collide
// (src/fsi/VariableViscosityDynamics.hh:151-172); BGK follows BGKdynamics::collide
// (src/basicDynamics/isoThermalDynamics.hh:329-340); TRT is Ginzburg's two-relaxation-
// time split around the same equilibrium (no reference counterpart).
template <class C, int COLL>
__device__ __forceinline__ void collide(C* f, const C* F, C omega, C omega_minus) {
    if (COLL == BIB_COLLISION_BGK_GUO_VOF) {
        const C rhoBar = rho_bar_seq(f);
        C u[3], j[3];
        velocity_with_force(f, F, u);
        const C rho = rhoBar + C(1);
        j[0] = rho * u[0];
        j[1] = rho * u[1];
        j[2] = rho * u[2];
        bgk_collision(f, rhoBar, j, omega, C(1) / (rhoBar + C(1)));
        guo_force(f, F, u, omega);
    } else if (COLL == BIB_COLLISION_BGK) {
        C rb, j[3];
        rho_bar_j(f, rb, j);
        bgk_collision(f, rb, j, omega, C(1) / (rb + C(1)));
    } else {
        C rb, j[3];
        rho_bar_j(f, rb, j);
        const C invRho = C(1) / (rb + C(1));
        const C jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
        f[0] = f[0] - omega * (f[0] - bgk_equilibrium<C>(0, rb, invRho, j, jSqr));
#pragma unroll
        for (int i = 1; i < 10; ++i) {
            const C ei = bgk_equilibrium<C>(i, rb, invRho, j, jSqr);
            const C eo = bgk_equilibrium<C>(i + 9, rb, invRho, j, jSqr);
            const C fp = C(0.5) * (f[i] + f[i + 9]), fm = C(0.5) * (f[i] - f[i + 9]);
            const C dp = omega * (fp - C(0.5) * (ei + eo));
            const C dm = omega_minus * (fm - C(0.5) * (ei - eo));
            f[i] = f[i] - dp - dm;
            f[i + 9] = f[i + 9] - dp + dm;
        }
    }
}

// Compact BGK + Guo collision for the reduced-precision paths.  Algebraically the same
// operator as collide<C, BGK_GUO_VOF>: with u = j/rho + F/2, rho = rhoBar + 1, the BGK
// equilibrium of J = rho u plus the Guo term of VariableViscosityDynamics.hh:47-129,
// t_i (1 - w/2) [3 (c_i - u).F + 9 (c_i.u)(c_i.F)], collapse to
//     f_i' = (1 - w) f_i + t_i [A + c_i.H + (c_i.u)(c_i.G)]
//     A = w rhoBar - 1.5 w rho u.u - 3 mu u.F,  H = 3 w rho u + 3 mu F,  G = 4.5 w rho u + 9 mu F,
// mu = 1 - w/2, evaluated once per opposite pair (i, i+9) (c_{i+9} = -c_i).  BGK without
// forcing is the same with F = 0 and u = j/rho.  The populations may carry a common scale S
// (FP16 storage keeps f-bar * S): moments are unscaled once, post-collision values come out
// in scaled units.  With `u_prev` non-null the velocity j/rho + F_prev/2 of the incoming
// state is returned as well (the reference's computeVelocity).
// c_i . (a, b, c) with the zero components left out: multiplications by 0 are not removed
// by the compiler under IEEE semantics (0 * inf is NaN), so they are not written.
__device__ __forceinline__ float cdot(int i, float a, float b, float c) {
    const float xa = cx(i) > 0 ? a : -a, yb = cy(i) > 0 ? b : -b, zc = cz(i) > 0 ? c : -c;
    if (cx(i) != 0) {
        if (cy(i) != 0) return xa + yb;
        if (cz(i) != 0) return xa + zc;
        return xa;
    }
    if (cy(i) != 0) return cz(i) != 0 ? yb + zc : yb;
    return cz(i) != 0 ? zc : 0.0f;
}

template <int COLL>
__device__ __forceinline__ void collide_compact(float* f, const float* F, float omega, float S, float invS,
                                                const float* Fprev, float* u_prev) {
    const float sxm = f[1] + f[4] + f[5] + f[6] + f[7];
    const float sxp = f[10] + f[13] + f[14] + f[15] + f[16];
    const float sym = f[2] + f[4] + f[8] + f[9] + f[14];
    const float syp = f[5] + f[11] + f[13] + f[17] + f[18];
    const float szm = f[3] + f[6] + f[8] + f[16] + f[18];
    const float szp = f[7] + f[9] + f[12] + f[15] + f[17];
    const float sx0 = f[0] + f[2] + f[3] + f[8] + f[9] + f[11] + f[12] + f[17] + f[18];
    const float rb = (sxm + sx0 + sxp) * invS;
    const float j0 = (sxp - sxm) * invS, j1 = (syp - sym) * invS, j2 = (szp - szm) * invS;
    const float invRho = 1.0f / (rb + 1.0f);
    if (u_prev) {
        u_prev[0] = fmaf(j0, invRho, 0.5f * Fprev[0]);
        u_prev[1] = fmaf(j1, invRho, 0.5f * Fprev[1]);
        u_prev[2] = fmaf(j2, invRho, 0.5f * Fprev[2]);
    }
    if (COLL == BIB_COLLISION_TRT) {
        // Two relaxation times around the BGK equilibrium of j: the symmetric part of each
        // pair (i, i+9) relaxes with omega, the antisymmetric part with omega_minus (passed
        // in F[0]); feq+ = t_i (rhoBar + 4.5 (c.j)^2 / rho - 1.5 j.j / rho), feq- = 3 t_i c.j.
        const float omm = F[0];
        const float base = rb - 1.5f * invRho * (j0 * j0 + j1 * j1 + j2 * j2);
        const float h = 4.5f * invRho;
        f[0] = fmaf(-omega, f[0] - (S * weight<float>(0)) * base, f[0]);
#pragma unroll
        for (int i = 1; i < 10; ++i) {
            const float cj = cdot(i, j0, j1, j2);
            const float tw = S * weight<float>(i);
            const float ep = tw * fmaf(h * cj, cj, base), em = tw * 3.0f * cj;
            const float dp = omega * (0.5f * (f[i] + f[i + 9]) - ep);
            const float dm = omm * (0.5f * (f[i] - f[i + 9]) - em);
            f[i] = f[i] - dp - dm;
            f[i + 9] = f[i + 9] - dp + dm;
        }
        return;
    }
    const bool forced = COLL == BIB_COLLISION_BGK_GUO_VOF;
    const float F0 = forced ? F[0] : 0.0f, F1 = forced ? F[1] : 0.0f, F2 = forced ? F[2] : 0.0f;
    const float u0 = fmaf(j0, invRho, 0.5f * F0), u1 = fmaf(j1, invRho, 0.5f * F1), u2 = fmaf(j2, invRho, 0.5f * F2);
    const float rho = rb + 1.0f;
    const float mu = 1.0f - 0.5f * omega;
    const float wr = omega * rho;
    const float A = omega * rb - 1.5f * wr * (u0 * u0 + u1 * u1 + u2 * u2) - 3.0f * mu * (u0 * F0 + u1 * F1 + u2 * F2);
    const float h3 = 3.0f * wr, m3 = 3.0f * mu, g45 = 4.5f * wr, m9 = 9.0f * mu;
    const float H0 = fmaf(h3, u0, m3 * F0), H1 = fmaf(h3, u1, m3 * F1), H2 = fmaf(h3, u2, m3 * F2);
    const float G0 = fmaf(g45, u0, m9 * F0), G1 = fmaf(g45, u1, m9 * F1), G2 = fmaf(g45, u2, m9 * F2);
    const float omo = 1.0f - omega;
    f[0] = fmaf(omo, f[0], (S * weight<float>(0)) * A);
#pragma unroll
    for (int i = 1; i < 10; ++i) {
        const float cu = cdot(i, u0, u1, u2), cG = cdot(i, G0, G1, G2), cH = cdot(i, H0, H1, H2);
        const float tw = S * weight<float>(i);
        const float P = tw * fmaf(cu, cG, A), M = tw * cH;
        f[i] = fmaf(omo, f[i], P + M);
        f[i + 9] = fmaf(omo, f[i + 9], P - M);
    }
}

__host__ __device__ inline int64_t wrap_index(int64_t i, int64_t n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

}  // namespace bib
