// Immersed-boundary kernels: delta interpolation of the lattice velocity to the
// membrane vertices, membrane forces + explicit vertex motion + area / volume /
// centre-of-mass update (one CTA per particle), and delta spreading of the vertex
// forces into the lattice force field.
//
// Vertices of all particles of a lattice are concatenated: positions (FP64, two
// buffers swapped every step), velocities and forces (FP64).
#include <cfloat>

#include "d3q19.cuh"

namespace bib {

namespace {

// ---------------------------------------------------------------- delta kernels
// RomaDirac<T,3>::eval and PeskinDirac<T,3>::eval(x), src/fsi/Dirac.h:27-31, 78-83
template <class W>
__device__ __forceinline__ W dirac_eval(int dirac, W x) {
    const W dx = fabs(x);
    if (dirac == BIB_DIRAC_PESKIN)
        return W(0.125) * (dx <= W(1) ? (W(3) - W(2) * dx + sqrt(W(1) + W(4) * dx * (W(1) - dx)))
                                      : (W(5) - W(2) * dx - sqrt(W(-7) + W(4) * dx * (W(3) - dx))));
    return (W(1) / W(6)) * (dx > W(0.5) ? (W(5) - W(3) * dx - sqrt(W(-3) * (W(1) - dx) * (W(1) - dx) + W(1)))
                                        : W(2) * (W(1) + sqrt(W(1) - W(3) * dx * dx)));
}

__device__ __forceinline__ double half_support(int dirac) { return dirac == BIB_DIRAC_PESKIN ? 2.0 : 1.5; }
__device__ __forceinline__ int support(int dirac) { return dirac == BIB_DIRAC_PESKIN ? 4 : 3; }

// Arithmetic1D::min_mod_diff (periodic) / plain difference, src/fsi/Periodicity.h:26-34, 93-96
__device__ __forceinline__ double axis_dist(int periodic, int N, double a, double b) {
    const double x = a - b;
    if (!periodic) return x;
    const double L = (double)N, Linv = 1.0 / L;
    return x - floor(x * Linv + 0.5) * L;
}

// Node classification of a single-block domain (ImmersedBoundaryDynamics.hh:46-66, 351-363):
// 1 bulk (support inside the domain), 2 envelope (general path), 0 outside.
__device__ int classify(const LatticeDesc& d, int dirac, const double* p) {
    const double h = half_support(dirac);
    const int N[3] = {d.nx, d.ny, d.nz};
    const int per[3] = {d.px, d.py, d.pz};
    const double shrink = 0.5 - h - DBL_EPSILON;
    bool in_env = true, in_bulk = true;
    for (int a = 0; a < 3; ++a) {
        const double top = (double)(N[a] - 1);
        const double elo = 0.0 - h, ehi = top + h;
        const double blo = 0.0 - shrink, bhi = top + shrink;
        in_env = in_env && fabs(axis_dist(per[a], N[a], 0.5 * (elo + ehi), p[a])) < 0.5 * (ehi - elo);
        in_bulk = in_bulk && fabs(axis_dist(per[a], N[a], 0.5 * (blo + bhi), p[a])) < 0.5 * (bhi - blo);
    }
    return !in_env ? 0 : (in_bulk ? 1 : 2);
}

// Arithmetic1D::remap_int(i, offset) with i0 = 0, Periodicity.h:106-110; returns a global
// index, or -1 for a non-periodic index outside the domain.
__device__ __forceinline__ int remap_global(int periodic, int N, int64_t i_local, int off) {
    int64_t g;
    if (periodic) {
        int64_t val = ((i_local + off + 100LL * N) % N) - off;
        if (val < 0) val += N;
        g = val + off;
    } else {
        g = i_local + off;
    }
    return (g < 0 || g >= N) ? -1 : (int)g;
}

// ---------------------------------------------------------------- interpolation
template <class T>
__device__ __forceinline__ void node_velocity(const LatticeDesc& d, const T* __restrict__ f,
                                              const typename Store<T>::F* __restrict__ F, int x, int y, int z,
                                              typename Store<T>::C* u) {
    using C = typename Store<T>::C;
    if (!d.py && d.wall_y == BIB_WALL_FD_VELOCITY && (y == 0 || y == d.ny - 1)) {
        const int side = y == 0 ? 0 : 1;
        u[0] = (C)d.wall_u[side][0];
        u[1] = (C)d.wall_u[side][1];
        u[2] = (C)d.wall_u[side][2];
        return;
    }
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    C fc[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) fc[i] = Store<T>::load(f + i * d.stride + k, d.inv_scale);
    C Fc[3] = {(C)F[k], (C)F[d.stride + k], (C)F[2 * d.stride + k]};
    velocity_with_force(fc, Fc, u);
}

template <class T>
__global__ void __launch_bounds__(128) k_interpolate(LatticeDesc d, IbDesc ib, int nvert, const double* __restrict__ pos,
                                                      const T* __restrict__ f, const typename Store<T>::F* __restrict__ F,
                                                      double* __restrict__ vel) {
    using C = typename Store<T>::C;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvert) return;
    const double p[3] = {pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
    double out[3] = {0.0, 0.0, 0.0};
    const int cls = classify(d, ib.dirac, p);
    if (cls != 0) {
        const int off = (int)ib.offset;
        const double pr[3] = {p[0] - ib.offset, p[1] - ib.offset, p[2] - ib.offset};
        const double h = half_support(ib.dirac);
        const int s = support(ib.dirac);
        int64_t lo[3];
        C w[3][4];
        for (int a = 0; a < 3; ++a) {
            lo[a] = (int64_t)ceil(pr[a] - h);
            for (int m = 0; m < s; ++m) w[a][m] = dirac_eval<C>(ib.dirac, (C)((double)(lo[a] + m) - pr[a]));
        }
        int gx[4], gy[4], gz[4];
        for (int m = 0; m < s; ++m) {
            gx[m] = remap_global(d.px, d.nx, lo[0] + m, off);
            gy[m] = remap_global(d.py, d.ny, lo[1] + m, off);
            gz[m] = remap_global(d.pz, d.nz, lo[2] + m, off);
        }
        C acc[3] = {C(0), C(0), C(0)};
        for (int a = 0; a < s; ++a) {
            if (gx[a] < 0) continue;
            for (int b = 0; b < s; ++b) {
                if (gy[b] < 0) continue;
                const C wxy = w[0][a] * w[1][b];
                for (int c = 0; c < s; ++c) {
                    if (gz[c] < 0) continue;
                    const C wt = wxy * w[2][c];
                    C u[3];
                    node_velocity<T>(d, f, F, gx[a], gy[b], gz[c], u);
                    acc[0] += wt * u[0];
                    acc[1] += wt * u[1];
                    acc[2] += wt * u[2];
                }
            }
        }
        out[0] = (double)acc[0];
        out[1] = (double)acc[1];
        out[2] = (double)acc[2];
    }
    vel[3 * v] = out[0];
    vel[3 * v + 1] = out[1];
    vel[3 * v + 2] = out[2];
}

// ---------------------------------------------------------------- spreading
template <class FT>
__global__ void __launch_bounds__(128) k_spread(LatticeDesc d, IbDesc ib, int nvert, const double* __restrict__ pos,
                                                 const double* __restrict__ force, FT* __restrict__ F) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvert) return;
    const double p[3] = {pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
    if (classify(d, ib.dirac, p) == 0) return;
    const int off = (int)ib.offset;
    const double pr[3] = {p[0] - ib.offset, p[1] - ib.offset, p[2] - ib.offset};
    const double h = half_support(ib.dirac);
    const int s = support(ib.dirac);
    int64_t lo[3];
    FT w[3][4];
    for (int a = 0; a < 3; ++a) {
        lo[a] = (int64_t)ceil(pr[a] - h);
        for (int m = 0; m < s; ++m) w[a][m] = dirac_eval<FT>(ib.dirac, (FT)((double)(lo[a] + m) - pr[a]));
    }
    int gx[4], gy[4], gz[4];
    for (int m = 0; m < s; ++m) {
        gx[m] = remap_global(d.px, d.nx, lo[0] + m, off);
        gy[m] = remap_global(d.py, d.ny, lo[1] + m, off);
        gz[m] = remap_global(d.pz, d.nz, lo[2] + m, off);
    }
    const FT fv[3] = {(FT)force[3 * v], (FT)force[3 * v + 1], (FT)force[3 * v + 2]};
    for (int a = 0; a < s; ++a) {
        if (gx[a] < 0) continue;
        for (int b = 0; b < s; ++b) {
            if (gy[b] < 0) continue;
            const FT wxy = w[0][a] * w[1][b];
            for (int c = 0; c < s; ++c) {
                if (gz[c] < 0) continue;
                const FT wt = wxy * w[2][c];
                const int64_t k = gx[a] + (int64_t)d.nx * (gy[b] + (int64_t)d.ny * gz[c]);
                atomicAdd(F + k, wt * fv[0]);
                atomicAdd(F + d.stride + k, wt * fv[1]);
                atomicAdd(F + 2 * d.stride + k, wt * fv[2]);
            }
        }
    }
}

// ---------------------------------------------------------------- membrane mechanics
template <class M>
struct V3 {
    M x, y, z;
};
template <class M>
__device__ __forceinline__ V3<M> mk3(M a, M b, M c) { return V3<M>{a, b, c}; }
template <class M>
__device__ __forceinline__ V3<M> operator+(V3<M> a, V3<M> b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class M>
__device__ __forceinline__ V3<M> operator-(V3<M> a, V3<M> b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class M>
__device__ __forceinline__ V3<M> operator*(M s, V3<M> a) { return mk3(s * a.x, s * a.y, s * a.z); }
template <class M>
__device__ __forceinline__ V3<M> operator/(V3<M> a, M s) { return mk3(a.x / s, a.y / s, a.z / s); }
template <class M>
__device__ __forceinline__ M dot3(V3<M> a, V3<M> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class M>
__device__ __forceinline__ M norm3(V3<M> a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
template <class M>
__device__ __forceinline__ V3<M> cross3(V3<M> a, V3<M> b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

template <class M>
__device__ __forceinline__ void acc_force(M* sf, int v, V3<M> f) {
    atomicAdd(sf + 3 * v, f.x);
    atomicAdd(sf + 3 * v + 1, f.y);
    atomicAdd(sf + 3 * v + 2, f.z);
}

// Vertex position relative to the particle's centre (exact FP64 subtraction, then
// rounding to M), so FP32 element arithmetic works on O(radius) numbers.
template <class M>
__device__ __forceinline__ V3<M> relpos(const double* pos, int v, const double* c) {
    return mk3<M>((M)(pos[3 * v] - c[0]), (M)(pos[3 * v + 1] - c[1]), (M)(pos[3 * v + 2] - c[2]));
}

// DeformableCapsuleParticle::compute_forces for one triangle, src/fsi/DeformableCapsule.hh:68-148
// (with the reference's c = l' sin(phi) / (l' sin(phi0)), line 96).
template <class M>
__device__ void capsule_triangle(const ParticleDev& P, int t, const double* pos, const double* c0, int skalak, M* sf) {
    const int i0 = P.tri[3 * t], i1 = P.tri[3 * t + 1], i2 = P.tri[3 * t + 2];
    const int id[3] = {i0, i1, i2};
    const V3<M> p0 = relpos<M>(pos, P.v0 + i0, c0), p1 = relpos<M>(pos, P.v0 + i1, c0), p2 = relpos<M>(pos, P.v0 + i2, c0);
    const V3<M> e0 = p1 - p0, e1 = p2 - p0;
    const V3<M> e0_0 = mk3<M>((M)(P.rest[3 * i1] - P.rest[3 * i0]), (M)(P.rest[3 * i1 + 1] - P.rest[3 * i0 + 1]),
                              (M)(P.rest[3 * i1 + 2] - P.rest[3 * i0 + 2]));
    const V3<M> e1_0 = mk3<M>((M)(P.rest[3 * i2] - P.rest[3 * i0]), (M)(P.rest[3 * i2 + 1] - P.rest[3 * i0 + 1]),
                              (M)(P.rest[3 * i2 + 2] - P.rest[3 * i0 + 2]));
    const M l = norm3(e0), lp = norm3(e1), l0 = norm3(e0_0), l0p = norm3(e1_0);
    const M e0e1 = dot3(e0, e1);
    const M sin_phi = norm3(cross3(e0, e1)) / (l * lp);
    const M cos_phi = e0e1 / (l * lp);
    const M sin_phi_0 = norm3(cross3(e0_0, e1_0)) / (l0 * l0p);
    const M cos_phi_0 = dot3(e0_0, e1_0) / (l0 * l0p);
    const M a = l / l0;
    const M b = (lp * cos_phi / l0p - l * cos_phi_0 / l0) / sin_phi_0;
    const M c = lp * sin_phi / (lp * sin_phi_0);
    const M D11 = (a * a - M(1)) / M(2);
    const M D22 = (b * b + c * c - M(1)) / M(2);
    const M D12 = a * b / M(2);
    const M I1 = M(2) * (D11 + D22);
    const M I2 = I1 + M(4) * (D11 * D22 - D12 * D12);
    const V3<M> zero = mk3<M>(0, 0, 0);
    const V3<M> gl[3] = {e0 / (-l), e0 / l, zero};
    const V3<M> glp[3] = {e1 / (-lp), zero, e1 / lp};
    const V3<M> gc[3] = {(M(-1) / (l * lp) + e0e1 / (l * l * l * lp)) * e0 + (M(-1) / (l * lp) + e0e1 / (l * lp * lp * lp)) * e1,
                         (M(1) / (l * lp)) * e1 - (e0e1 / (l * l * l * lp)) * e0,
                         (M(1) / (l * lp)) * e0 - (e0e1 / (l * lp * lp * lp)) * e1};
    const M s0sq = sin_phi_0 * sin_phi_0;
    const M G = (M)P.prm[BIB_P_G], Cc = (M)P.prm[BIB_P_C];
    const M pref = -G / M(2) * (M)P.tri_area[t];
    for (int i = 0; i < 3; ++i) {
        const V3<M> gD11 = (l / (l0 * l0)) * gl[i];
        const V3<M> gD22 = (M(1) / s0sq) * ((lp / (l0p * l0p) - l * cos_phi * cos_phi_0 / (l0 * l0p)) * glp[i] +
                                            (l * (cos_phi_0 * cos_phi_0) / (l0 * l0) - lp * cos_phi * cos_phi_0 / (l0p * l0)) * gl[i] -
                                            (l * lp * cos_phi_0 / (l0 * l0p)) * gc[i]);
        const V3<M> gD12 = (M(1) / (M(2) * l0p * sin_phi_0)) *
                           ((lp * cos_phi / l0p - M(2) * l * cos_phi_0 / l0) * gl[i] + (l * cos_phi / l0p) * glp[i] +
                            (l * lp / l0p) * gc[i]);
        const V3<M> gI1 = M(2) * (gD11 + gD22);
        const V3<M> gI2 = (M(2) + M(4) * D22) * gD11 + (M(2) + M(4) * D11) * gD22 - (M(8) * D12) * gD12;
        V3<M> fv;
        if (skalak) fv = pref * ((I1 + M(1)) * gI1 + (Cc * I2 - M(1)) * gI2);
        else fv = pref * (gI1 - (M(1) / ((M(1) + I2) * (M(1) + I2))) * gI2);
        acc_force(sf, id[i], fv);
    }
}

// RBCParticle link term (WLC + POW), src/fsi/RBCParticle.hh:148-169 with
// RBCParameters::in_plane_ks_kp (RBCParticle.hh:27-44), m = 2, x0 = 1/2.2.
template <class M>
__device__ void rbc_link(const ParticleDev& P, int l, const double* pos, const double* c0, M* sf) {
    const double x0 = 1. / 2.2;
    const double ks_c1 = 0.25 * (6. * x0 + (3 * x0 * x0 - 2 * x0 * x0 * x0) / ((1 - x0) * (1 - x0)));
    const double ks_c2 = x0 / (2. * (1 - x0) * (1 - x0) * (1 - x0)) + 0.25 * (1. - 1. / ((1 - x0) * (1 - x0)));
    const double l0 = P.link_len[l];
    const double kp_c1 = -1. / (l0 * l0), kp_c2 = 3. / (l0 * l0);
    const double G_lhs = 4. * l0 * P.prm[BIB_P_SHEAR_MODULUS] / sqrt(3.0);
    const double den = ks_c1 * kp_c2 - ks_c2 * kp_c1;
    const M ks = (M)(-kp_c1 * G_lhs / den), kp = (M)(ks_c1 * G_lhs / den);
    const int a = P.links[2 * l], b = P.links[2 * l + 1];
    const V3<M> dv = relpos<M>(pos, P.v0 + a, c0) - relpos<M>(pos, P.v0 + b, c0);
    const M L = norm3(dv);
    const M x = L / (M)(l0 * 2.2);
    const M df = M(-0.25) * ks * (M(6) * x + (M(3) * x * x - M(2) * x * x * x) / ((M(1) - x) * (M(1) - x))) + kp / (L * L);
    const V3<M> fv = (df / L) * dv;
    acc_force(sf, a, fv);
    acc_force(sf, b, M(-1) * fv);
}

// RBCParticle triangle terms: global + local area and volume penalties,
// src/fsi/RBCParticle.hh:175-213 with tri::triangle_area_and_gradient and
// tri::grad_signed_volume (TriangleUtils.h:58-120).  The volume gradient is
// translation invariant on a closed surface, so it is taken relative to the centre.
template <class M>
__device__ void rbc_triangle(const ParticleDev& P, int t, const double* pos, const double* c0, double area, double volume,
                             M* sf) {
    const int i0 = P.tri[3 * t], i1 = P.tri[3 * t + 1], i2 = P.tri[3 * t + 2];
    const V3<M> v0 = relpos<M>(pos, P.v0 + i0, c0), v1 = relpos<M>(pos, P.v0 + i1, c0), v2 = relpos<M>(pos, P.v0 + i2, c0);
    const M v01v11 = v0.y - v1.y, v02v22 = v0.z - v2.z, v02v12 = v0.z - v1.z;
    const M v01v21 = v0.y - v2.y, v00v20 = v0.x - v2.x, v00v10 = v0.x - v1.x;
    const M a = v01v11 * v02v22 - v02v12 * v01v21;
    const M b = v02v12 * v00v20 - v00v10 * v02v22;
    const M c = v00v10 * v01v21 - v01v11 * v00v20;
    const M la = M(0.5) * sqrt(a * a + b * b + c * c);
    const M denom = M(1) / (M(4) * la);
    const V3<M> g0 = mk3<M>((b * (v2.z - v1.z) + c * (v1.y - v2.y)) * denom, (a * (v1.z - v2.z) + c * (v2.x - v1.x)) * denom,
                            (a * (v2.y - v1.y) + b * (v1.x - v2.x)) * denom);
    const V3<M> g1 = mk3<M>((b * v02v22 + c * (v2.y - v0.y)) * denom, (a * (v2.z - v0.z) + c * v00v20) * denom,
                            (a * v01v21 + b * (v2.x - v0.x)) * denom);
    const V3<M> g2 = mk3<M>((b * (v1.z - v0.z) + c * v01v11) * denom, (a * v02v12 + c * (v1.x - v0.x)) * denom,
                            (a * (v1.y - v0.y) + b * v00v10) * denom);
    // penalty differences in FP64
    const double A0 = P.A0;
    M df_area = (M)(P.prm[BIB_P_K_AREA_GLOBAL] * (A0 - area) / A0);
    df_area += (M)P.prm[BIB_P_K_AREA_LOCAL] * ((M)P.tri_area[t] - la) / (M)P.tri_area[t];
    acc_force(sf, i0, df_area * g0);
    acc_force(sf, i1, df_area * g1);
    acc_force(sf, i2, df_area * g2);
    const M df_vol = (M)(P.prm[BIB_P_K_VOLUME] * (P.prm[BIB_P_VOL_DESIRED] - volume) / P.prm[BIB_P_VOL_DESIRED]);
    acc_force(sf, i0, (df_vol / M(6)) * cross3(v1, v2));
    acc_force(sf, i1, (df_vol / M(6)) * cross3(v2, v0));
    acc_force(sf, i2, (df_vol / M(6)) * cross3(v0, v1));
}

// Dihedral bending of one adjacent-triangle pair, src/fsi/RBCParticle.hh:217-246 with
// tri::grad_angle_between_pair (TriangleUtils.h:139-164).
template <class M>
__device__ void rbc_pair(const ParticleDev& P, int p, const double* pos, const double* c0, M* sf) {
    const int* q = P.pairs + 4 * p;
    const V3<M> v0 = relpos<M>(pos, P.v0 + q[0], c0), v1 = relpos<M>(pos, P.v0 + q[1], c0);
    const V3<M> v2 = relpos<M>(pos, P.v0 + q[2], c0), v3 = relpos<M>(pos, P.v0 + q[3], c0);
    const V3<M> e0 = v1 - v0, e1 = v2 - v0, e2 = v3 - v0;
    const M e1n = norm3(e1);
    const V3<M> e1u = e1 / e1n;
    const V3<M> n1 = cross3(e0, e1), n2 = cross3(e1, e2);
    const M n1n = norm3(n1), n2n = norm3(n2);
    const V3<M> n1u = n1 / n1n, n2u = n2 / n2n;
    const M cos_t = dot3(n1u, n2u);
    const M sin_t = (dot3(n1 - n2, v1 - v3) > M(0) ? M(1) : M(-1)) * norm3(cross3(n1u, n2u));
    const M pref = (M)P.prm[BIB_P_K_BEND] * (-(M)P.pair_cs[2 * p] * sin_t + (M)P.pair_cs[2 * p + 1] * cos_t);
    acc_force(sf, q[0], pref * ((dot3(e1u, e1 - e2) / n2n) * n2u + (dot3(e1u, e1 - e0) / n1n) * n1u));
    acc_force(sf, q[1], pref * ((-e1n / n1n) * n1u));
    acc_force(sf, q[2], pref * ((dot3(e1u, e2) / n2n) * n2u + (dot3(e1u, e0) / n1n) * n1u));
    acc_force(sf, q[3], pref * ((-e1n / n2n) * n2u));
}

template <class T>
__device__ __forceinline__ T block_sum(T v, T* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    T r = T(0);
    if (threadIdx.x < 32) {
        r = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : T(0);
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;  // valid in thread 0
}

// One CTA per particle: forces at X_n (ParticleBase3D::reset_forces + compute_forces),
// X_{n+1} = X_n + U_n (DeformableParticle3D::move_vertices, DeformableParticle3D.hh:26-51),
// area / volume / area-weighted centre (update(), :54-82) and the periodic centre-of-mass
// remap (ParticleBase3D::map_center_of_mass_to_periodic_grid, ParticleBase.hh:111-136).
template <class M>
__global__ void __launch_bounds__(256) k_membrane(LatticeDesc d, const ParticleDev* __restrict__ parts,
                                                   const double* __restrict__ pos, double* __restrict__ pos_next,
                                                   const double* __restrict__ vel, double* __restrict__ force,
                                                   double* __restrict__ stats) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    M* sf = reinterpret_cast<M*>(smem_raw);
    __shared__ double red[32];
    __shared__ double com_new[3];
    const ParticleDev& P = parts[blockIdx.x];
    double* st = stats + STATS * blockIdx.x;
    const double area = st[0], volume = st[1];
    // FP64 element arithmetic uses absolute positions as the reference does; reduced
    // precision works relative to the centre of mass.
    const bool rel = sizeof(M) < sizeof(double);
    const double c0[3] = {rel ? st[2] : 0.0, rel ? st[3] : 0.0, rel ? st[4] : 0.0};
    for (int i = threadIdx.x; i < 3 * P.nv; i += blockDim.x) sf[i] = M(0);
    __syncthreads();
    if (P.model == BIB_MODEL_CAPSULE_NEOHOOKEAN || P.model == BIB_MODEL_CAPSULE_SKALAK || P.model == BIB_MODEL_SKALAK_BENDING) {
        const int skalak = P.model != BIB_MODEL_CAPSULE_NEOHOOKEAN;
        for (int t = threadIdx.x; t < P.nt; t += blockDim.x) capsule_triangle<M>(P, t, pos, c0, skalak, sf);
    }
    if (P.model == BIB_MODEL_RBC_WLCPOW) {
        for (int l = threadIdx.x; l < P.nl; l += blockDim.x) rbc_link<M>(P, l, pos, c0, sf);
    }
    if (P.model == BIB_MODEL_RBC_WLCPOW || P.model == BIB_MODEL_SKALAK_BENDING) {
        for (int t = threadIdx.x; t < P.nt; t += blockDim.x) rbc_triangle<M>(P, t, pos, c0, area, volume, sf);
        for (int p = threadIdx.x; p < P.np; p += blockDim.x) rbc_pair<M>(P, p, pos, c0, sf);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * P.nv; i += blockDim.x) {
        const int64_t g = 3LL * P.v0 + i;
        force[g] = (double)sf[i];
        pos_next[g] = pos[g] + vel[g];
    }
    __syncthreads();
    // update(): area, signed volume and area-weighted centroid of X_{n+1}
    double sa = 0, sv = 0, scx = 0, scy = 0, scz = 0;
    for (int t = threadIdx.x; t < P.nt; t += blockDim.x) {
        const double* a = pos_next + 3LL * (P.v0 + P.tri[3 * t]);
        const double* b = pos_next + 3LL * (P.v0 + P.tri[3 * t + 1]);
        const double* c = pos_next + 3LL * (P.v0 + P.tri[3 * t + 2]);
        const V3<double> A = mk3(a[0], a[1], a[2]), B = mk3(b[0], b[1], b[2]), Cv = mk3(c[0], c[1], c[2]);
        const double dA = norm3(cross3(B - A, Cv - A)) * 0.5;
        sa += dA;
        sv += dot3(A, cross3(B, Cv)) / 6.;
        const V3<double> cen = (A + B + Cv) / 3.0;
        scx += cen.x * dA;
        scy += cen.y * dA;
        scz += cen.z * dA;
    }
    sa = block_sum(sa, red);
    __syncthreads();
    sv = block_sum(sv, red);
    __syncthreads();
    scx = block_sum(scx, red);
    __syncthreads();
    scy = block_sum(scy, red);
    __syncthreads();
    scz = block_sum(scz, red);
    if (threadIdx.x == 0) {
        double com[3] = {scx / sa, scy / sa, scz / sa};
        const int N[3] = {d.nx, d.ny, d.nz};
        const int per[3] = {d.px, d.py, d.pz};
        double np_[3];
        for (int a = 0; a < 3; ++a) {
            np_[a] = com[a];
            if (per[a]) {
                const double L = (double)N[a], Linv = 1. / L;
                np_[a] = com[a] - L * floor((com[a] - (-0.5)) * Linv);
            }
            com_new[a] = np_[a] - com[a];  // delta
        }
        st[0] = sa;
        st[1] = sv;
        st[2] = np_[0];
        st[3] = np_[1];
        st[4] = np_[2];
    }
    __syncthreads();
    if (com_new[0] != 0.0 || com_new[1] != 0.0 || com_new[2] != 0.0) {
        for (int i = threadIdx.x; i < P.nv; i += blockDim.x) {
            const int64_t g = 3LL * (P.v0 + i);
            pos_next[g] += com_new[0];
            pos_next[g + 1] += com_new[1];
            pos_next[g + 2] += com_new[2];
        }
    }
}

}  // namespace

size_t membrane_smem_bytes(int max_nv) { return (size_t)3 * max_nv * sizeof(double); }

void configure_membrane_kernel(size_t smem) {
    cudaFuncSetAttribute(k_membrane<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_membrane<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

void launch_interpolate(const Lattice& L, cudaStream_t s) {
    if (L.nvert == 0) return;
    const unsigned g = (L.nvert + 127) / 128;
    const double* pos = L.pos[L.pcur];
    if (L.storage == BIB_STORAGE_F64)
        k_interpolate<double><<<g, 128, 0, s>>>(L.d, L.ib, L.nvert, pos, (const double*)L.f[L.cur], (const double*)L.F, L.vel);
    else if (L.storage == BIB_STORAGE_F32)
        k_interpolate<float><<<g, 128, 0, s>>>(L.d, L.ib, L.nvert, pos, (const float*)L.f[L.cur], (const float*)L.F, L.vel);
    else
        k_interpolate<__half><<<g, 128, 0, s>>>(L.d, L.ib, L.nvert, pos, (const __half*)L.f[L.cur], (const float*)L.F, L.vel);
}

void launch_membrane(const Lattice& L, cudaStream_t s) {
    const int np = (int)L.parts.size();
    if (np == 0) return;
    if (L.storage == BIB_STORAGE_F64)
        k_membrane<double><<<np, 256, L.membrane_smem, s>>>(L.d, L.pdev, L.pos[L.pcur], L.pos[1 - L.pcur], L.vel, L.force, L.stats);
    else
        k_membrane<float><<<np, 256, L.membrane_smem / 2, s>>>(L.d, L.pdev, L.pos[L.pcur], L.pos[1 - L.pcur], L.vel, L.force, L.stats);
}

void launch_spread(const Lattice& L, cudaStream_t s) {
    if (L.nvert == 0) return;
    const unsigned g = (L.nvert + 127) / 128;
    const double* pos = L.pos[L.pcur];
    if (L.storage == BIB_STORAGE_F64) k_spread<double><<<g, 128, 0, s>>>(L.d, L.ib, L.nvert, pos, L.force, (double*)L.F);
    else k_spread<float><<<g, 128, 0, s>>>(L.d, L.ib, L.nvert, pos, L.force, (float*)L.F);
}

}  // namespace bib
