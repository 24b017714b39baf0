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
// get_rhoBar_j (partial sums), src/latticeBoltzmann/momentTemplates3D.h:350-423
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

// Collision of one cell, every kernel and every precision.  BGK_GUO_VOF is
// GuoExternalForceVOFDynamics::collide (src/fsi/VariableViscosityDynamics.hh:151-172): with
// u = j/rho + F/2, rho = rhoBar + 1, the BGK equilibrium of J = rho u
// (bgk_ma2_collision_base, src/latticeBoltzmann/dynamicsTemplates3D.h:770-838) plus the Guo term of
// VariableViscosityDynamics.hh:47-129,
// t_i (1 - w/2) [3 (c_i - u).F + 9 (c_i.u)(c_i.F)], collapse to
//     f_i' = (1 - w) f_i + t_i [A + c_i.H + (c_i.u)(c_i.G)]
//     A = w rhoBar - 1.5 w rho u.u - 3 mu u.F,  H = 3 w rho u + 3 mu F,  G = 4.5 w rho u + 9 mu F,
// mu = 1 - w/2, evaluated once per opposite pair (i, i+9) (c_{i+9} = -c_i).  BGK without
// forcing is the same with F = 0 and u = j/rho (BGKdynamics::collide,
// src/basicDynamics/isoThermalDynamics.hh:329-340); TRT is Ginzburg's two-relaxation-time split
// around the same equilibrium (no reference counterpart).  The populations may carry a common scale S
// (FP16 storage keeps f-bar * S): moments are unscaled once, post-collision values come out
// in scaled units.  With `u_prev` non-null the velocity j/rho + F_prev/2 of the incoming
// state is returned as well (the reference's computeVelocity).
// c_i . (a, b, c) with the zero components left out: multiplications by 0 are not removed
// by the compiler under IEEE semantics (0 * inf is NaN), so they are not written.
template <class C>
__device__ __forceinline__ C cdot(int i, C a, C b, C c) {
    const C xa = cx(i) > 0 ? a : -a, yb = cy(i) > 0 ? b : -b, zc = cz(i) > 0 ? c : -c;
    if (cx(i) != 0) {
        if (cy(i) != 0) return xa + yb;
        if (cz(i) != 0) return xa + zc;
        return xa;
    }
    if (cy(i) != 0) return cz(i) != 0 ? yb + zc : yb;
    return cz(i) != 0 ? zc : C(0);
}
__device__ __forceinline__ float fmac(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmac(double a, double b, double c) { return fma(a, b, c); }

// Moments of the incoming state: rhoBar, j and 1/rho, unscaled.
template <class C>
struct CellMoments {
    C rb, j0, j1, j2, invRho;
};
template <class C>
__device__ __forceinline__ CellMoments<C> moments_compact(const C* f, C invS) {
    const C sxm = f[1] + f[4] + f[5] + f[6] + f[7];
    const C sxp = f[10] + f[13] + f[14] + f[15] + f[16];
    const C sym = f[2] + f[4] + f[8] + f[9] + f[14];
    const C syp = f[5] + f[11] + f[13] + f[17] + f[18];
    const C szm = f[3] + f[6] + f[8] + f[16] + f[18];
    const C szp = f[7] + f[9] + f[12] + f[15] + f[17];
    const C sx0 = f[0] + f[2] + f[3] + f[8] + f[9] + f[11] + f[12] + f[17] + f[18];
    CellMoments<C> m;
    m.rb = (sxm + sx0 + sxp) * invS;
    m.j0 = (sxp - sxm) * invS;
    m.j1 = (syp - sym) * invS;
    m.j2 = (szp - szm) * invS;
    m.invRho = C(1) / (m.rb + C(1));
    return m;
}

// The velocity j/rho + F_prev/2 of the incoming state (the reference's computeVelocity).
template <class C>
__device__ __forceinline__ void velocity_compact(const CellMoments<C>& m, const C* Fprev, C* u) {
    u[0] = fmac(m.j0, m.invRho, C(0.5) * Fprev[0]);
    u[1] = fmac(m.j1, m.invRho, C(0.5) * Fprev[1]);
    u[2] = fmac(m.j2, m.invRho, C(0.5) * Fprev[2]);
}

// Relaxation of one cell from its moments (scaled populations in, scaled populations out).
template <class C, int COLL>
__device__ __forceinline__ void relax_compact(C* f, const C* F, C omega, C S, const CellMoments<C>& m) {
    const C rb = m.rb, j0 = m.j0, j1 = m.j1, j2 = m.j2, invRho = m.invRho;
    if (COLL == BIB_COLLISION_TRT) {
        // Two relaxation times around the BGK equilibrium of j: the symmetric part of each
        // pair (i, i+9) relaxes with omega, the antisymmetric part with omega_minus (passed
        // in F[0]); feq+ = t_i (rhoBar + 4.5 (c.j)^2 / rho - 1.5 j.j / rho), feq- = 3 t_i c.j.
        // Collected per pair: f_i' = a f_i + b f_i+9 + (w feq+ + w- feq-) and f_i+9' = a f_i+9 +
        // b f_i + (w feq+ - w- feq-), with a = 1 - (w + w-)/2 and b = (w- - w)/2.
        const C omm = F[0];
        const C base = rb - C(1.5) * invRho * (j0 * j0 + j1 * j1 + j2 * j2);
        const C h = C(4.5) * invRho;
        const C a = C(1) - C(0.5) * (omega + omm), b = C(0.5) * (omm - omega);
        const C oS = omega * S, mS3 = C(3) * omm * S;
        f[0] = fmac(C(1) - omega, f[0], (oS * weight<C>(0)) * base);
#pragma unroll
        for (int i = 1; i < 10; ++i) {
            const C cj = cdot<C>(i, j0, j1, j2);
            const C P = (oS * weight<C>(i)) * fmac(h * cj, cj, base), M = (mS3 * weight<C>(i)) * cj;
            const C fi = f[i], fo = f[i + 9];
            f[i] = fmac(a, fi, fmac(b, fo, P + M));
            f[i + 9] = fmac(a, fo, fmac(b, fi, P - M));
        }
        return;
    }
    const bool forced = COLL == BIB_COLLISION_BGK_GUO_VOF;
    const C F0 = forced ? F[0] : C(0), F1 = forced ? F[1] : C(0), F2 = forced ? F[2] : C(0);
    const C u0 = fmac(j0, invRho, C(0.5) * F0), u1 = fmac(j1, invRho, C(0.5) * F1), u2 = fmac(j2, invRho, C(0.5) * F2);
    const C rho = rb + C(1);
    const C mu = C(1) - C(0.5) * omega;
    const C wr = omega * rho;
    const C A = omega * rb - C(1.5) * wr * (u0 * u0 + u1 * u1 + u2 * u2) - C(3) * mu * (u0 * F0 + u1 * F1 + u2 * F2);
    const C h3 = C(3) * wr, m3 = C(3) * mu, g45 = C(4.5) * wr, m9 = C(9) * mu;
    const C H0 = fmac(h3, u0, m3 * F0), H1 = fmac(h3, u1, m3 * F1), H2 = fmac(h3, u2, m3 * F2);
    const C G0 = fmac(g45, u0, m9 * F0), G1 = fmac(g45, u1, m9 * F1), G2 = fmac(g45, u2, m9 * F2);
    const C omo = C(1) - omega;
    f[0] = fmac(omo, f[0], (S * weight<C>(0)) * A);
#pragma unroll
    for (int i = 1; i < 10; ++i) {
        const C cu = cdot<C>(i, u0, u1, u2), cG = cdot<C>(i, G0, G1, G2), cH = cdot<C>(i, H0, H1, H2);
        const C tw = S * weight<C>(i);
        const C P = tw * fmac(cu, cG, A), M = tw * cH;
        f[i] = fmac(omo, f[i], P + M);
        f[i + 9] = fmac(omo, f[i + 9], P - M);
    }
}

template <class C, int COLL>
__device__ __forceinline__ void collide_compact(C* f, const C* F, C omega, C S, C invS, const C* Fprev, C* u_prev) {
    const CellMoments<C> m = moments_compact<C>(f, invS);
    if (u_prev) velocity_compact<C>(m, Fprev, u_prev);
    relax_compact<C, COLL>(f, F, omega, S, m);
}

// The compact operators at unit scale (FP64 / FP32 populations held as f-bar): omega_minus is the
// TRT rate of the antisymmetric parts, unused otherwise.
template <class C, int COLL>
__device__ __forceinline__ void collide_unscaled(C* f, const C* F, C omega, C omega_minus) {
    if (COLL == BIB_COLLISION_TRT) {
        const C Fm[3] = {omega_minus, C(0), C(0)};
        collide_compact<C, COLL>(f, Fm, omega, C(1), C(1), nullptr, nullptr);
    } else {
        collide_compact<C, COLL>(f, F, omega, C(1), C(1), nullptr, nullptr);
    }
}

__host__ __device__ inline int64_t wrap_index(int64_t i, int64_t n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

}  // namespace bib
