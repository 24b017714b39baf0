// Immersed-boundary kernels: delta interpolation of the lattice velocity to the
// membrane vertices, membrane forces + explicit vertex motion + area / volume /
// centre-of-mass update (one CTA per particle), and delta spreading of the vertex
// forces into the lattice force field.
//
// Vertices of all particles of a lattice are concatenated: positions (FP64, two
// buffers swapped every step), velocities and forces (FP64).
#include <algorithm>
#include <cfloat>

#include <cub/device/device_radix_sort.cuh>

#include "lattice_common.cuh"

namespace bib {

namespace {

// Reduced-precision arithmetic: the FP32 element and weight evaluations use the hardware's
// approximate square root, reciprocal and division (a few ulp); FP64 keeps the IEEE
// operations of the reference's expressions.
__device__ __forceinline__ float fast_sqrt(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double fast_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float fast_rcp(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double fast_rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float fast_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double fast_div(double a, double b) { return a / b; }

// ---------------------------------------------------------------- delta kernels
// RomaDirac<T,3>::eval and PeskinDirac<T,3>::eval(x), src/fsi/Dirac.h:27-31, 78-83
template <class W>
__device__ __forceinline__ W dirac_eval(int dirac, W x) {
    const W dx = fabs(x);
    if (dirac == BIB_DIRAC_PESKIN)
        return W(0.125) * (dx <= W(1) ? (W(3) - W(2) * dx + fast_sqrt(W(1) + W(4) * dx * (W(1) - dx)))
                                      : (W(5) - W(2) * dx - fast_sqrt(W(-7) + W(4) * dx * (W(3) - dx))));
    return (W(1) / W(6)) * (dx > W(0.5) ? (W(5) - W(3) * dx - fast_sqrt(W(-3) * (W(1) - dx) * (W(1) - dx) + W(1)))
                                        : W(2) * (W(1) + fast_sqrt(W(1) - W(3) * dx * dx)));
}

__device__ __forceinline__ double half_support(int dirac) { return dirac == BIB_DIRAC_PESKIN ? 2.0 : 1.5; }
__device__ __forceinline__ int support(int dirac) { return dirac == BIB_DIRAC_PESKIN ? 4 : 3; }

// Node classes of a single-block domain (ImmersedBoundaryDynamics.hh:46-66, 351-363): a
// vertex is in the envelope when, on every axis, the min-mod distance from the domain
// centre (N - 1)/2 is below the half width (N - 1)/2 + h (the bulk / envelope split only
// selects between two interpolators with the same result here).  On a periodic axis the
// min-mod distance is at most N/2 < (N - 1)/2 + h, so only walled axes can put a vertex
// outside.  Non-finite positions are outside.
__device__ __forceinline__ bool inside_envelope(const LatticeDesc& d, int dirac, const double* p) {
    const double h = half_support(dirac);
    const int N[3] = {d.nx, d.ny, d.nz};
    const int per[3] = {d.px, d.py, d.pz};
    bool in = true;
    for (int a = 0; a < 3; ++a) {
        if (per[a]) {
            in = in && isfinite(p[a]);
        } else {
            const double top = (double)(N[a] - 1);
            const double elo = 0.0 - h, ehi = top + h;
            in = in && fabs(0.5 * (elo + ehi) - p[a]) < 0.5 * (ehi - elo);
        }
    }
    return in;
}

// Positive remainder of x modulo N; the division is only taken more than a period away.
__device__ __forceinline__ int pmod(int64_t x, int N) {
    if (x >= 0 && x < N) return (int)x;
    if (x < 0 && x >= -(int64_t)N) return (int)(x + N);
    if (x >= N && x < 2LL * N) return (int)(x - N);
    const int64_t r = x % N;
    return (int)(r < 0 ? r + N : r);
}

// Arithmetic1D::remap_int(i, offset) with i0 = 0, Periodicity.h:106-110; returns a global
// index, or -1 for a non-periodic index outside the domain.
__device__ __forceinline__ int remap_global(int periodic, int N, int64_t i_local, int off) {
    int64_t g;
    if (periodic) {
        int val = pmod(i_local + off, N) - off;
        if (val < 0) val += N;
        g = (int64_t)val + off;
    } else {
        g = i_local + off;
    }
    return (g < 0 || g >= N) ? -1 : (int)g;
}

// First support node of one axis as the spreading records it for the sparse force reset: on a
// periodic axis reduced to one period (remap_global of lo + m is unchanged), so that it fits 32
// bits; on a walled axis a vertex inside the envelope is within h + 1 of the domain.
__device__ __forceinline__ int record_lo(int periodic, int N, int64_t lo, int off) {
    return periodic ? pmod(lo + off, N) - off : (int)lo;
}

// Delta weight of support node lo + m on one axis, phi(lo + m - x) with lo = ceil(x - h).
// FP32 weights take the FP64 offset lo - x and add m in FP32.
template <class W>
__device__ __forceinline__ W axis_weight(int dirac, int64_t lo, double x, int m) {
    if (sizeof(W) == sizeof(double)) return dirac_eval<W>(dirac, (W)((double)(lo + m) - x));
    return dirac_eval<W>(dirac, (W)((double)lo - x) + (W)m);
}
template <class W, int S>
__device__ __forceinline__ int64_t axis_weights(double x, W* w) {
    constexpr int dirac = S == 4 ? BIB_DIRAC_PESKIN : BIB_DIRAC_ROMA;
    const int64_t lo = (int64_t)ceil(x - half_support(dirac));
#pragma unroll
    for (int m = 0; m < S; ++m) w[m] = axis_weight<W>(dirac, lo, x, m);
    return lo;
}

// Windows of up to four consecutive cells of one x-row of one force component, added with
// one or two aligned float4 atomics (the field rows start 16-byte aligned: the component
// stride is a multiple of 128 cells).  Slots outside the window add zero.
__device__ __forceinline__ float window_select(const float* x, int j, int o, int s) {
    float r = 0.0f;
#pragma unroll
    for (int m = 0; m < 4; ++m)
        if (m < s && j - o == m) r = x[m];
    return r;
}
__device__ __forceinline__ void red_window(float* row, int64_t k0, const float* v, int s) {
    const int64_t kq = k0 & ~(int64_t)3;
    const int o = (int)(k0 - kq);
    float4* q = reinterpret_cast<float4*>(row + kq);
    atomicAdd(q, make_float4(window_select(v, 0, o, s), window_select(v, 1, o, s), window_select(v, 2, o, s),
                             window_select(v, 3, o, s)));
    if (o + s > 4)
        atomicAdd(q + 1, make_float4(window_select(v, 4, o, s), window_select(v, 5, o, s), window_select(v, 6, o, s),
                                     window_select(v, 7, o, s)));
}
// One cell of the velocity field ((ux, uy, uz, 0) per cell), one or two vector loads.
template <class C>
struct U3 {
    C x, y, z;
};
__device__ __forceinline__ U3<float> load_u(const float* u, int64_t k) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(u) + k);
    return U3<float>{v.x, v.y, v.z};
}
__device__ __forceinline__ U3<double> load_u(const double* u, int64_t k) {
    const double2* q = reinterpret_cast<const double2*>(u) + 2 * k;
    const double2 a = __ldg(q), b = __ldg(q + 1);
    return U3<double>{a.x, a.y, b.x};
}
__device__ __forceinline__ U3<float> load_u(const __half* u, int64_t k) {  // FP16 population storage
    const uint2 v = __ldg(reinterpret_cast<const uint2*>(u) + k);
    const float2 ab = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
    return U3<float>{ab.x, ab.y, __low2float(*reinterpret_cast<const __half2*>(&v.y))};
}
// Compute type of an interpolation from the velocity field's storage type.
template <class UT>
struct InterpC {
    using type = float;
};
template <>
struct InterpC<double> {
    using type = double;
};

// ---------------------------------------------------------------- pipe boundary
// PipeBoundary::distance_to_boundary (fsi/Boundary.h:158-161) minus the kernel's half support:
// the weight of the supplied kernel against the 2-point TopHat near the wall (>= 1: the
// supplied kernel alone, <= 0: the TopHat alone, _interpolation.hh:181-230, _forces.hh:192-237)
__device__ __forceinline__ double pipe_weight(const IbDesc& ib, const double* p, double h) {
    const double dy = p[1] - ib.pipe_y0, dz = p[2] - ib.pipe_z0;
    return ib.pipe_r - sqrt(dy * dy + dz * dz) - h;
}

// TopHatDirac<T,3> (Dirac.h:47-64): support 2, weight 1 - |x| per axis; the 2 x 2 x 2 nodes
// in GeneralInterpolator / GeneralSpreading order.  mode 0 gathers u into acc, mode 1 adds
// w * fv into the force field.
template <class C, class UT>
__device__ __forceinline__ void tophat_interp(const LatticeDesc& d, const IbDesc& ib, const double* p, const UT* u, C* acc) {
    const int off = (int)ib.offset;
    int64_t lo[3];
    C w[3][2];
    for (int a = 0; a < 3; ++a) {
        const double x = p[a] - ib.offset;
        lo[a] = (int64_t)ceil(x - 1.0);
        w[a][0] = (C)(1. - fabs((double)lo[a] - x));
        w[a][1] = (C)(1. - fabs((double)(lo[a] + 1) - x));
    }
    for (int a = 0; a < 2; ++a) {
        const int gx = remap_global(d.px, d.nx, lo[0] + a, off);
        if (gx < 0) continue;
        for (int b = 0; b < 2; ++b) {
            const int gy = remap_global(d.py, d.ny, lo[1] + b, off);
            if (gy < 0) continue;
            const C wxy = w[0][a] * w[1][b];
            for (int c = 0; c < 2; ++c) {
                const int gz = remap_global(d.pz, d.nz, lo[2] + c, off);
                if (gz < 0) continue;
                const C wt = wxy * w[2][c];
                const U3<C> uc = load_u(u, gx + (int64_t)d.nx * (gy + (int64_t)d.ny * gz));
                acc[0] += wt * uc.x;
                acc[1] += wt * uc.y;
                acc[2] += wt * uc.z;
            }
        }
    }
}
template <class FT>
__device__ __forceinline__ void tophat_spread(const LatticeDesc& d, const IbDesc& ib, const double* p, const FT* fv, FT* F) {
    const int off = (int)ib.offset;
    int64_t lo[3];
    FT w[3][2];
    for (int a = 0; a < 3; ++a) {
        const double x = p[a] - ib.offset;
        lo[a] = (int64_t)ceil(x - 1.0);
        w[a][0] = (FT)(1. - fabs((double)lo[a] - x));
        w[a][1] = (FT)(1. - fabs((double)(lo[a] + 1) - x));
    }
    for (int a = 0; a < 2; ++a) {
        const int gx = remap_global(d.px, d.nx, lo[0] + a, off);
        if (gx < 0) continue;
        for (int b = 0; b < 2; ++b) {
            const int gy = remap_global(d.py, d.ny, lo[1] + b, off);
            if (gy < 0) continue;
            const FT wxy = w[0][a] * w[1][b];
            for (int c = 0; c < 2; ++c) {
                const int gz = remap_global(d.pz, d.nz, lo[2] + c, off);
                if (gz < 0) continue;
                const FT wt = wxy * w[2][c];
                FT* q = F + gx + (int64_t)d.nx * (gy + (int64_t)d.ny * gz);
                atomicAdd(q, wt * fv[0]);
                atomicAdd(q + d.stride, wt * fv[1]);
                atomicAdd(q + 2 * d.stride, wt * fv[2]);
            }
        }
    }
}

// DeformableParticle3D::move_vertices(boundary) (DeformableParticle3D.hh:26-51) with
// PipeBoundary::trace_ray / get_normal (Boundary.h:164-187, 245-249): a step that crosses the
// wall is reflected about the normal at the crossing.
__device__ __forceinline__ void pipe_move(const IbDesc& ib, const double* old, const double* v, double* x) {
    const double y1 = old[1] - ib.pipe_y0, y2 = x[1] - ib.pipe_y0, z1 = old[2] - ib.pipe_z0, z2 = x[2] - ib.pipe_z0;
    const double a = (y2 - y1) * (y2 - y1) + (z2 - z1) * (z2 - z1);
    const double b = y1 * (y2 - y1) + z1 * (z2 - z1);
    const double c = y1 * y1 + z1 * z1 - ib.pipe_r * ib.pipe_r;
    const double disc = b * b - c * a;
    if (disc < 0. || fabs(a) < 10 * DBL_EPSILON) return;
    const double bOverA = -b / a, sqrtDisc = sqrt(disc) / a;
    double t = bOverA - sqrtDisc;
    if (!(t >= 0. && t <= 1.)) {
        t = bOverA + sqrtDisc;
        if (!(t >= 0. && t <= 1.)) return;
    }
    for (int k = 0; k < 3; ++k) x[k] = old[k] + t * v[k];
    const double ny_ = x[1] - ib.pipe_y0, nz_ = x[2] - ib.pipe_z0;
    const double nn = sqrt(0.0 * 0.0 + ny_ * ny_ + nz_ * nz_);
    const double n[3] = {0.0 / nn, ny_ / nn, nz_ / nn};
    const double s2 = 2. * (v[0] * n[0] + v[1] * n[1] + v[2] * n[2]);
    for (int k = 0; k < 3; ++k) x[k] += (v[k] - s2 * n[k]) * (1. - t);
}

// ---------------------------------------------------------------- interpolation
// Interpolation of the velocity field (written by the collide-and-stream kernel or the
// velocity kernel) to every vertex, followed by the explicit Euler move
// X_{n+1} = X_n + U_n (DeformableParticle3D::move_vertices, DeformableParticle3D.hh:26-51).
// Classes and index arithmetic follow interpolate_impl with the Bulk / General
// interpolators, ImmersedBoundaryDynamics_interpolation.hh:13-153.
// One thread per vertex.  BATCH: the vertex numbering runs over the lattices of a batch and
// each thread looks its lattice's view up through vinst; otherwise v1 is the lattice.
// FOLD (sparse force reset): the velocity field holds j/rho + body/2, and the vertex velocity
// adds the share of the previous step's force, sum of w (Fold - body) / 2 over the support
// nodes off the finite-difference wall rows (whose velocity is the wall's); the sum of the two
// is the interpolation of j/rho + Fold/2, the reference's computeVelocity field.
template <class UT, int S, bool FOLD = false>
__device__ __forceinline__ void interpolate_move_vertex(const IbView& V, int v) {
    using C = typename InterpC<UT>::type;  // also the force field's type
    static_assert(S == 3 || S == 4, "Roma (3) or Peskin (4) support");
    const LatticeDesc& d = V.d;
    const IbDesc& ib = V.ib;
    const double* __restrict__ pos = V.pos;
    double* __restrict__ pos_next = V.pos_next;
    const UT* __restrict__ u = static_cast<const UT*>(V.u);
    double* __restrict__ vel = V.vel;
    const double p[3] = {pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
    double out[3] = {0.0, 0.0, 0.0};
    if (inside_envelope(d, ib.dirac, p)) {
        const int off = (int)ib.offset;
        constexpr int s = S;
        int64_t lo[3];
        C w[3][4];
        for (int a = 0; a < 3; ++a) lo[a] = axis_weights<C, S>(p[a] - ib.offset, w[a]);
        int gx[4], gy[4], gz[4];
#pragma unroll
        for (int m = 0; m < s; ++m) {
            gx[m] = remap_global(d.px, d.nx, lo[0] + m, off);
            gy[m] = remap_global(d.py, d.ny, lo[1] + m, off);
            gz[m] = remap_global(d.pz, d.nz, lo[2] + m, off);
        }
        int64_t yo[4], zo[4];  // row offsets of the support nodes
#pragma unroll
        for (int m = 0; m < s; ++m) {
            yo[m] = (int64_t)gy[m] * d.nx;
            zo[m] = (int64_t)gz[m] * d.ny * d.nx;
        }
        C acc[3] = {C(0), C(0), C(0)};
        C facc[3] = {C(0), C(0), C(0)};
        const C* __restrict__ Fo = static_cast<const C*>(V.Fold);
        const C body[3] = {(C)d.body[0], (C)d.body[1], (C)d.body[2]};
#pragma unroll
        for (int a = 0; a < s; ++a) {
            if (gx[a] < 0) continue;
#pragma unroll
            for (int b = 0; b < s; ++b) {
                if (gy[b] < 0) continue;
                const C wxy = w[0][a] * w[1][b];
                const int64_t col = gx[a] + yo[b];
                const bool fd_row = FOLD && fd_wall_node(d, gy[b]);
#pragma unroll
                for (int c = 0; c < s; ++c) {
                    if (gz[c] < 0) continue;
                    const C wt = wxy * w[2][c];
                    const U3<C> uc = load_u(u, col + zo[c]);
                    acc[0] += wt * uc.x;
                    acc[1] += wt * uc.y;
                    acc[2] += wt * uc.z;
                    if (FOLD && !fd_row) {
                        const int64_t k = col + zo[c];
                        facc[0] += wt * (__ldg(Fo + k) - body[0]);
                        facc[1] += wt * (__ldg(Fo + d.stride + k) - body[1]);
                        facc[2] += wt * (__ldg(Fo + 2 * d.stride + k) - body[2]);
                    }
                }
            }
        }
        out[0] = (double)(FOLD ? acc[0] + C(0.5) * facc[0] : acc[0]);
        out[1] = (double)(FOLD ? acc[1] + C(0.5) * facc[1] : acc[1]);
        out[2] = (double)(FOLD ? acc[2] + C(0.5) * facc[2] : acc[2]);
    }
    if (ib.has_pipe && inside_envelope(d, ib.dirac, p)) {
        const double w = pipe_weight(ib, p, S == 4 ? 2.0 : 1.5);
        if (w < 1) {  // near the wall: blend with (or switch to) the TopHat kernel
            C t[3] = {C(0), C(0), C(0)};
            tophat_interp<C, UT>(d, ib, p, u, t);
            for (int k = 0; k < 3; ++k) out[k] = w <= 0 ? (double)t[k] : (1. - w) * (double)t[k] + w * out[k];
        }
    }
    vel[3 * v] = out[0];
    vel[3 * v + 1] = out[1];
    vel[3 * v + 2] = out[2];
    double xn[3] = {p[0] + out[0], p[1] + out[1], p[2] + out[2]};
    if (ib.has_pipe) pipe_move(ib, p, out, xn);
    pos_next[3 * v] = xn[0];
    pos_next[3 * v + 1] = xn[1];
    pos_next[3 * v + 2] = xn[2];
}

// 9 CTAs of 128 threads per SM (at most 56 registers): measured 2 % faster than 8 on the
// 400-cell channel (the kernel waits on its gathers; more warps hide more of that)
template <class UT, int S, bool BATCH, bool FOLD = false>
__global__ void __launch_bounds__(128, 9) k_interpolate_move(IbView v1, const IbView* __restrict__ views,
                                                           const int* __restrict__ vinst, int nvert) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nvert) return;
    const IbView& V = BATCH ? views[vinst[g]] : v1;
    interpolate_move_vertex<UT, S, FOLD>(V, BATCH ? g - V.vbase : (V.order ? V.order[g] : g));
}

// Sparse force reset: F := body force at the support nodes the last spreading into F recorded
// (one thread per vertex and (y, z) row of its support).  Along x the stores cover the aligned
// float4 words around the row's s nodes: a cell of such a word outside the support holds the body
// force already or lies in the support of another vertex, which is reset in the same launch.
template <int S>
__global__ void __launch_bounds__(128) k_force_clear(LatticeDesc d, IbDesc ib, int nvert, const int4* __restrict__ lo,
                                                      float* __restrict__ F) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nvert * S * S) return;
    const int v = (int)(t / (S * S)), r = (int)(t - (int64_t)v * S * S);
    const int4 l = lo[v];
    if (!l.w) return;
    const int off = (int)ib.offset;
    const int gy = remap_global(d.py, d.ny, (int64_t)l.y + r / S, off);
    const int gz = remap_global(d.pz, d.nz, (int64_t)l.z + r % S, off);
    if (gy < 0 || gz < 0) return;
    const int64_t row = (int64_t)d.nx * (gy + (int64_t)d.ny * gz);
    const float b[3] = {(float)d.body[0], (float)d.body[1], (float)d.body[2]};
    const int gx0 = remap_global(d.px, d.nx, (int64_t)l.x, off);
    const int gxl = remap_global(d.px, d.nx, (int64_t)l.x + S - 1, off);
    if (gx0 >= 0 && gxl == gx0 + S - 1) {
        // the row's nodes are contiguous: the float4 words from gx0 down to 4 to gxl
        const int64_t k0 = (row + gx0) & ~(int64_t)3, k1 = (row + gxl) & ~(int64_t)3;
        for (int q = 0; q < 3; ++q) {
            float4* p = reinterpret_cast<float4*>(F + q * d.stride);
            for (int64_t k = k0; k <= k1; k += 4) p[k >> 2] = make_float4(b[q], b[q], b[q], b[q]);
        }
        return;
    }
#pragma unroll
    for (int m = 0; m < S; ++m) {
        const int gx = remap_global(d.px, d.nx, (int64_t)l.x + m, off);
        if (gx < 0) continue;
        for (int q = 0; q < 3; ++q) F[q * d.stride + row + gx] = b[q];
    }
}

// ---------------------------------------------------------------- spreading
template <class FT, int S>
__device__ __forceinline__ void spread_vertex(const IbView& V, int v) {
    static_assert(S == 3 || S == 4, "Roma (3) or Peskin (4) support");
    const LatticeDesc& d = V.d;
    const IbDesc& ib = V.ib;
    const double* __restrict__ pos = V.pos;
    const double* __restrict__ force = V.force;
    FT* __restrict__ F = static_cast<FT*>(V.F);
    const double p[3] = {pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
    if (!inside_envelope(d, ib.dirac, p)) {
        if (V.spread_lo) V.spread_lo[v] = make_int4(0, 0, 0, 0);
        return;
    }
    const int off = (int)ib.offset;
    constexpr int s = S;
    if (V.spread_lo) {
        constexpr double h = S == 4 ? 2.0 : 1.5;
        V.spread_lo[v] = make_int4(record_lo(d.px, d.nx, (int64_t)ceil(p[0] - ib.offset - h), off),
                                   record_lo(d.py, d.ny, (int64_t)ceil(p[1] - ib.offset - h), off),
                                   record_lo(d.pz, d.nz, (int64_t)ceil(p[2] - ib.offset - h), off), 1);
    }
    FT fscale = FT(1);
    if (ib.has_pipe) {
        const double wp = pipe_weight(ib, p, S == 4 ? 2.0 : 1.5);
        if (wp < 1) {  // near the wall: the TopHat takes the share 1 - w of the force
            FT* Fw = static_cast<FT*>(V.F);
            const FT ft[3] = {(FT)(force[3 * v] * (wp <= 0 ? 1.0 : 1. - wp)),
                              (FT)(force[3 * v + 1] * (wp <= 0 ? 1.0 : 1. - wp)),
                              (FT)(force[3 * v + 2] * (wp <= 0 ? 1.0 : 1. - wp))};
            tophat_spread<FT>(d, ib, p, ft, Fw);
            if (wp <= 0) return;
            fscale = (FT)wp;
        }
    }
    int64_t lo[3];
    FT w[3][4];
    for (int a = 0; a < 3; ++a) lo[a] = axis_weights<FT, S>(p[a] - ib.offset, w[a]);
    int gx[4], gy[4], gz[4];
#pragma unroll
    for (int m = 0; m < s; ++m) {
        gx[m] = remap_global(d.px, d.nx, lo[0] + m, off);
        gy[m] = remap_global(d.py, d.ny, lo[1] + m, off);
        gz[m] = remap_global(d.pz, d.nz, lo[2] + m, off);
    }
    int64_t yo[4], zo[4];
#pragma unroll
    for (int m = 0; m < s; ++m) {
        yo[m] = (int64_t)gy[m] * d.nx;
        zo[m] = (int64_t)gz[m] * d.ny * d.nx;
    }
    const FT fv[3] = {fscale == FT(1) ? (FT)force[3 * v] : (FT)(force[3 * v] * (double)fscale),
                      fscale == FT(1) ? (FT)force[3 * v + 1] : (FT)(force[3 * v + 1] * (double)fscale),
                      fscale == FT(1) ? (FT)force[3 * v + 2] : (FT)(force[3 * v + 2] * (double)fscale)};
    if (sizeof(FT) == sizeof(float) && gx[s - 1] == gx[0] + s - 1) {
        // FP32 field and no periodic wrap along x inside the support: each (y, z) row of
        // each component receives one window of s values through one or two float4 atomics
        float* Ff = reinterpret_cast<float*>(F);
#pragma unroll
        for (int b = 0; b < s; ++b) {
            if (gy[b] < 0) continue;
#pragma unroll
            for (int c = 0; c < s; ++c) {
                if (gz[c] < 0) continue;
                const FT wyz = w[1][b] * w[2][c];
                const int64_t k0 = gx[0] + yo[b] + zo[c];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    float vals[4];
                    for (int m = 0; m < 4; ++m) vals[m] = m < s ? (float)((w[0][m] * wyz) * fv[q]) : 0.0f;
                    red_window(Ff + q * d.stride, k0, vals, s);
                }
            }
        }
        return;
    }
#pragma unroll
    for (int a = 0; a < s; ++a) {
        if (gx[a] < 0) continue;
#pragma unroll
        for (int b = 0; b < s; ++b) {
            if (gy[b] < 0) continue;
            const FT wxy = w[0][a] * w[1][b];
            FT* col = F + gx[a] + yo[b];
#pragma unroll
            for (int c = 0; c < s; ++c) {
                if (gz[c] < 0) continue;
                const FT wt = wxy * w[2][c];
                FT* q = col + zo[c];
                atomicAdd(q, wt * fv[0]);
                atomicAdd(q + d.stride, wt * fv[1]);
                atomicAdd(q + 2 * d.stride, wt * fv[2]);
            }
        }
    }
}

template <class FT, int S, bool BATCH>
__global__ void __launch_bounds__(128) k_spread(IbView v1, const IbView* __restrict__ views, const int* __restrict__ vinst,
                                                 int nvert) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nvert) return;
    const IbView& V = BATCH ? views[vinst[g]] : v1;
    spread_vertex<FT, S>(V, BATCH ? g - V.vbase : g);
}

// Two lanes per vertex (FP32 field, Roma support, no pipe, no wrap along x inside the support):
// the lanes of a pair add the two float4 words of a window that straddles a 16-byte boundary in
// the same instruction, so that both words go out in one request when they share a 128-byte line
// (the spreading is bound by the count of its requests: 0.0950 -> 0.0835 ms on the 400-cell
// channel against one lane issuing both words).  Same products as spread_vertex.
__device__ __forceinline__ void spread_vertex_pair(const IbView& V, int v, int half) {
    const LatticeDesc& d = V.d;
    const IbDesc& ib = V.ib;
    const double p[3] = {V.pos[3 * v], V.pos[3 * v + 1], V.pos[3 * v + 2]};
    if (!inside_envelope(d, ib.dirac, p)) {
        if (V.spread_lo && half == 0) V.spread_lo[v] = make_int4(0, 0, 0, 0);
        return;
    }
    const int off = (int)ib.offset;
    int64_t lo[3];
    float w[3][4];
#pragma unroll
    for (int a = 0; a < 3; ++a) lo[a] = axis_weights<float, 3>(p[a] - ib.offset, w[a]);
    int gx[3], gy[3], gz[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        gx[m] = remap_global(d.px, d.nx, lo[0] + m, off);
        gy[m] = remap_global(d.py, d.ny, lo[1] + m, off);
        gz[m] = remap_global(d.pz, d.nz, lo[2] + m, off);
    }
    if (ib.has_pipe || gx[2] != gx[0] + 2) {
        if (half == 0) spread_vertex<float, 3>(V, v);
        return;
    }
    if (V.spread_lo && half == 0)
        V.spread_lo[v] = make_int4(record_lo(d.px, d.nx, (int64_t)ceil(p[0] - ib.offset - 1.5), off),
                                   record_lo(d.py, d.ny, (int64_t)ceil(p[1] - ib.offset - 1.5), off),
                                   record_lo(d.pz, d.nz, (int64_t)ceil(p[2] - ib.offset - 1.5), off), 1);
    const float fv[3] = {(float)V.force[3 * v], (float)V.force[3 * v + 1], (float)V.force[3 * v + 2]};
    float* F = static_cast<float*>(V.F);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        if (gy[b] < 0) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (gz[c] < 0) continue;
            const float wyz = w[1][b] * w[2][c];
            const int64_t k0 = gx[0] + (int64_t)gy[b] * d.nx + (int64_t)gz[c] * d.ny * d.nx;
            const int64_t kq = k0 & ~(int64_t)3;
            const int o = (int)(k0 - kq);
            const bool go = half == 0 || o + 3 > 4;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                float vals[4];
#pragma unroll
                for (int m = 0; m < 4; ++m) vals[m] = m < 3 ? (float)((w[0][m] * wyz) * fv[q]) : 0.0f;
                const int j = half * 4;
                const float4 val = make_float4(window_select(vals, j, o, 3), window_select(vals, j + 1, o, 3),
                                               window_select(vals, j + 2, o, 3), window_select(vals, j + 3, o, 3));
                if (go) atomicAdd(reinterpret_cast<float4*>(F + q * d.stride + kq) + half, val);
            }
        }
    }
}

__global__ void __launch_bounds__(128) k_spread_pairs(IbView v1, int nvert) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = g >> 1;
    if (v >= nvert) return;
    spread_vertex_pair(v1, v, g & 1);
}

// Deterministic spreading.  Every (vertex, stencil node) pair becomes an entry keyed by its
// target cell; a stable radix sort groups the entries of a cell in vertex order, and one
// thread per cell sums its contributions in that order onto the body force already in F.
// The result does not depend on scheduling (the atomic path does, in its last bits).
// Entries that spread nowhere carry the key n (one past the last cell), so the sort needs
// only ceil(log2(n + 1)) key bits.
__host__ __device__ inline int key_bits(int64_t n) {
    int b = 1;
    while (((int64_t)1 << b) <= n) ++b;
    return b;
}

__global__ void __launch_bounds__(128) k_spread_keys(LatticeDesc d, IbDesc ib, int nvert, const double* __restrict__ pos,
                                                      uint32_t* __restrict__ keys, uint32_t* __restrict__ ids,
                                                      int4* __restrict__ lo_out) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvert) return;
    const int s = support(ib.dirac), s3 = s * s * s;
    const double p[3] = {pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
    const bool inside = inside_envelope(d, ib.dirac, p);
    const int off = (int)ib.offset;
    const double h = half_support(ib.dirac);
    int64_t lo[3];
    for (int a = 0; a < 3; ++a) lo[a] = (int64_t)ceil(p[a] - ib.offset - h);
    if (lo_out)
        lo_out[v] = inside ? make_int4(record_lo(d.px, d.nx, lo[0], off), record_lo(d.py, d.ny, lo[1], off),
                                       record_lo(d.pz, d.nz, lo[2], off), 1)
                           : make_int4(0, 0, 0, 0);
    for (int m = 0; m < s3; ++m) {
        const int a = m / (s * s), b = (m / s) % s, c = m % s;
        const int gx = remap_global(d.px, d.nx, lo[0] + a, off);
        const int gy = remap_global(d.py, d.ny, lo[1] + b, off);
        const int gz = remap_global(d.pz, d.nz, lo[2] + c, off);
        const bool ok = inside && gx >= 0 && gy >= 0 && gz >= 0;
        keys[(int64_t)v * s3 + m] = ok ? (uint32_t)(gx + (int64_t)d.nx * (gy + (int64_t)d.ny * gz)) : (uint32_t)d.n;
        ids[(int64_t)v * s3 + m] = (uint32_t)((int64_t)v * s3 + m);
    }
}

template <class FT>
__global__ void __launch_bounds__(128) k_spread_reduce(LatticeDesc d, IbDesc ib, int64_t nentries,
                                                        const uint32_t* __restrict__ keys, const uint32_t* __restrict__ ids,
                                                        const double* __restrict__ pos, const double* __restrict__ force,
                                                        FT* __restrict__ F) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= nentries) return;
    const uint32_t key = keys[p];
    if (key == (uint32_t)d.n || (p > 0 && keys[p - 1] == key)) return;  // not the head of a cell's run
    const int s = support(ib.dirac), s3 = s * s * s;
    const double h = half_support(ib.dirac);
    FT acc[3] = {F[key], F[d.stride + key], F[2 * d.stride + key]};
    for (int64_t q = p; q < nentries && keys[q] == key; ++q) {
        const uint32_t e = ids[q];
        const int v = (int)(e / s3), m = (int)(e % s3);
        const int a = m / (s * s), b = (m / s) % s, c = m % s;
        const double pr[3] = {pos[3 * v] - ib.offset, pos[3 * v + 1] - ib.offset, pos[3 * v + 2] - ib.offset};
        FT w[3];
        const int sel[3] = {a, b, c};
        for (int ax = 0; ax < 3; ++ax) {
            const int64_t lo = (int64_t)ceil(pr[ax] - h);
            w[ax] = axis_weight<FT>(ib.dirac, lo, pr[ax], sel[ax]);
        }
        const FT wt = (w[0] * w[1]) * w[2];
        acc[0] += wt * (FT)force[3 * v];
        acc[1] += wt * (FT)force[3 * v + 1];
        acc[2] += wt * (FT)force[3 * v + 2];
    }
    F[key] = acc[0];
    F[d.stride + key] = acc[1];
    F[2 * d.stride + key] = acc[2];
}

// ---------------------------------------------------------------- interaction forces
// MorsePotential::eval / SpringPotential::operator() (fsi/Potentials.h:29-71), FP64
__device__ __forceinline__ double potential_eval(const PotentialDev& p, double d) {
    if (p.kind == BIB_POTENTIAL_MORSE) {
        if (d < 0) d = 0.0;
        const double x = exp(p.beta * (p.r0 - d));
        return 2 * p.beta * p.strength * x * (x - 1);
    }
    if (p.kind == BIB_POTENTIAL_SPRING) return (p.r0 - d) * p.strength;
    return 0.0;
}

// Sum of the wall-interaction decorators on a vertex at p (WallInteraction::apply_force,
// ForceDecorator.hh:25-32, with ParallelPlatesBoundary, Boundary.h:305-365): for the nearer
// plate at distance dist <= r0, force -= phi(dist) * outward normal.
__device__ __forceinline__ void wall_force(const Interactions& I, const double* p, double* f) {
    f[0] = f[1] = f[2] = 0.0;
    for (int w = 0; w < I.nwall; ++w) {
        const int a = I.wall_axis[w];
        if (a == 3) {  // PipeBoundary: distance_to_boundary and get_normal, Boundary.h:158-161, 245-249
            const double dy = p[1] - I.wall_lo[w], dz = p[2] - I.wall_hi[w];
            const double rr = sqrt(dy * dy + dz * dz);
            const double dist = I.wall_r[w] - rr;
            if (dist <= I.wall[w].r0) {
                // the normal (0, dy, dz) / |.| of get_normal: on the axis (rr = 0) every component,
                // the x one included, is 0/0, as in the reference
                const double phi = potential_eval(I.wall[w], dist);
                f[0] -= phi * (0.0 / rr);
                f[1] -= phi * (dy / rr);
                f[2] -= phi * (dz / rr);
            }
            continue;
        }
        const double r = p[a], lo = I.wall_lo[w], hi = I.wall_hi[w];
        const bool lower = r < 0.5 * (lo + hi);
        const double dist = lower ? r - lo : hi - r;
        if (dist <= I.wall[w].r0) {
            const double phi = potential_eval(I.wall[w], dist);
            f[a] -= lower ? -phi : phi;
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
__device__ __forceinline__ M norm3(V3<M> a) { return fast_sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// a / s: one approximate reciprocal in FP32, the three IEEE divisions in FP64
template <class M>
__device__ __forceinline__ V3<M> div3(V3<M> a, M s) {
    if constexpr (sizeof(M) == sizeof(float)) return fast_rcp(s) * a;
    else return a / s;
}
template <class M>
__device__ __forceinline__ V3<M> cross3(V3<M> a, V3<M> b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Element force consumers: AtomicSink accumulates every corner force into shared memory
// (order of summation left to the hardware); GatherSink keeps the contributions to one
// vertex, in the order the elements are visited (deterministic).
template <class M>
struct AtomicSink {
    M* sf;
    __device__ __forceinline__ void operator()(int v, V3<M> f) const {
        atomicAdd(sf + 3 * v, f.x);
        atomicAdd(sf + 3 * v + 1, f.y);
        atomicAdd(sf + 3 * v + 2, f.z);
    }
};
template <class M>
struct GatherSink {
    int target;
    V3<M> acc;
    __device__ __forceinline__ void operator()(int v, V3<M> f) {
        if (v == target) acc = acc + f;
    }
};

// Vertex positions as the element kernels see them.  GlobalPos reads the FP64 positions
// (relative to c, exact FP64 subtraction, then rounding to M); SharedPos reads a copy of
// the particle's relative positions staged in shared memory.
template <class M>
struct GlobalPos {
    const double* pos;  // particle's first vertex
    double c[3];
    __device__ __forceinline__ V3<M> operator()(int v) const {
        return mk3<M>((M)(pos[3 * v] - c[0]), (M)(pos[3 * v + 1] - c[1]), (M)(pos[3 * v + 2] - c[2]));
    }
};
template <class M>
struct SharedPos {
    const M* sp;
    __device__ __forceinline__ V3<M> operator()(int v) const { return mk3<M>(sp[3 * v], sp[3 * v + 1], sp[3 * v + 2]); }
};

// Per-particle constants of the element kernels, evaluated once per thread in the
// element precision M (the FP64 expressions are the reference's, so M = double gives the
// same values as evaluating them per element).
template <class M>
struct MemCoef {
    M G, C;            // capsule shear modulus and area-dilation ratio
    M kb;              // bending modulus
    M k_area_local;
    M df_area_global;  // k_area_global (A0 - A) / A0
    M df_vol6;         // k_volume (V_desired - V) / V_desired / 6
};
template <class M>
__device__ __forceinline__ MemCoef<M> mem_coef(const ParticleDev& P, double area, double volume) {
    MemCoef<M> k;
    k.G = (M)P.prm[BIB_P_G];
    k.C = (M)P.prm[BIB_P_C];
    k.kb = (M)P.prm[BIB_P_K_BEND];
    k.k_area_local = (M)P.prm[BIB_P_K_AREA_LOCAL];
    k.df_area_global = (M)(P.prm[BIB_P_K_AREA_GLOBAL] * (P.A0 - area) / P.A0);
    k.df_vol6 = (M)(P.prm[BIB_P_K_VOLUME] * (P.prm[BIB_P_VOL_DESIRED] - volume) / P.prm[BIB_P_VOL_DESIRED]) / M(6);
    return k;
}
template <class M>
__device__ __forceinline__ M tri_area_of(const ParticleDev& P, int t) {
    return sizeof(M) == sizeof(double) ? (M)P.tri_area[t] : (M)P.tri_area_f[t];
}
template <class M>
__device__ __forceinline__ M pair_c(const ParticleDev& P, int p, int k) {
    return sizeof(M) == sizeof(double) ? (M)P.pair_cs[2 * p + k] : (M)P.pair_cs_f[2 * p + k];
}

// DeformableCapsuleParticle::compute_forces for one triangle, src/fsi/DeformableCapsule.hh:68-148
// (with the reference's c = l' sin(phi) / (l' sin(phi0)), line 96).  The rest-state lengths
// and angle come from the FP64 rest mesh (M = double) or its FP32 copies.
template <class M, class PS, class Sink>
__device__ void capsule_triangle(const ParticleDev& P, int t, int4 ti, const PS& ps, int skalak, const MemCoef<M>& k,
                                 Sink& sk) {
    const int i0 = ti.x, i1 = ti.y, i2 = ti.z;
    const int id[3] = {i0, i1, i2};
    const V3<M> p0 = ps(i0), p1 = ps(i1), p2 = ps(i2);
    const V3<M> e0 = p1 - p0, e1 = p2 - p0;
    M l0, l0p, sin_phi_0, cos_phi_0;
    if (sizeof(M) == sizeof(double)) {
        const V3<M> e0_0 = mk3<M>((M)(P.rest[3 * i1] - P.rest[3 * i0]), (M)(P.rest[3 * i1 + 1] - P.rest[3 * i0 + 1]),
                                  (M)(P.rest[3 * i1 + 2] - P.rest[3 * i0 + 2]));
        const V3<M> e1_0 = mk3<M>((M)(P.rest[3 * i2] - P.rest[3 * i0]), (M)(P.rest[3 * i2 + 1] - P.rest[3 * i0 + 1]),
                                  (M)(P.rest[3 * i2 + 2] - P.rest[3 * i0 + 2]));
        l0 = norm3(e0_0);
        l0p = norm3(e1_0);
        sin_phi_0 = norm3(cross3(e0_0, e1_0)) / (l0 * l0p);
        cos_phi_0 = dot3(e0_0, e1_0) / (l0 * l0p);
    } else {
        const float4 r = reinterpret_cast<const float4*>(P.tri_rest_f)[t];
        l0 = (M)r.x;
        l0p = (M)r.y;
        cos_phi_0 = (M)r.z;
        sin_phi_0 = (M)r.w;
    }
    if constexpr (sizeof(M) == sizeof(float)) {
        // The same forces with the corner-independent scalars gathered: every gradient of
        // D11, D22, D12 (hence of I1, I2) is a combination of the corner gradients of
        // l, l' and cos(phi) (gl, glp, gc below), so f_i = pref (Cl gl_i + Cp glp_i + Cq gc_i);
        // reciprocals are taken once.
        const M l = norm3(e0), lp = norm3(e1);
        const M e0e1 = dot3(e0, e1), cr = norm3(cross3(e0, e1));
        const M rl = fast_rcp(l), rlp = fast_rcp(lp), rl0 = fast_rcp(l0), rl0p = fast_rcp(l0p), rs0 = fast_rcp(sin_phi_0);
        const M rllp = rl * rlp;
        const M sin_phi = cr * rllp, cos_phi = e0e1 * rllp;
        const M a = l * rl0;
        const M b = (lp * cos_phi * rl0p - l * cos_phi_0 * rl0) * rs0;
        const M c = sin_phi * rs0;
        const M D11 = (a * a - M(1)) * M(0.5);
        const M D22 = (b * b + c * c - M(1)) * M(0.5);
        const M D12 = a * b * M(0.5);
        const M I1 = M(2) * (D11 + D22);
        const M I2 = I1 + M(4) * (D11 * D22 - D12 * D12);
        M w1, w2;
        if (skalak) {
            w1 = I1 + M(1);
            w2 = k.C * I2 - M(1);
        } else {
            const M q = M(1) + I2;
            w1 = M(1);
            w2 = -fast_rcp(q * q);
        }
        const M A11 = l * rl0 * rl0, s2 = rs0 * rs0;
        const M k22p = s2 * (lp * rl0p * rl0p - l * cos_phi * cos_phi_0 * rl0 * rl0p);
        const M k22l = s2 * (l * cos_phi_0 * cos_phi_0 * rl0 * rl0 - lp * cos_phi * cos_phi_0 * rl0p * rl0);
        const M k22c = -s2 * l * lp * cos_phi_0 * rl0 * rl0p;
        const M k12 = M(0.5) * rl0p * rs0;
        const M k12l = k12 * (lp * cos_phi * rl0p - M(2) * l * cos_phi_0 * rl0);
        const M k12p = k12 * l * cos_phi * rl0p, k12c = k12 * l * lp * rl0p;
        const M al = M(2) + M(4) * D22, be = M(2) + M(4) * D11, ga = M(8) * D12;
        const M Cl = M(2) * w1 * (A11 + k22l) + w2 * (al * A11 + be * k22l - ga * k12l);
        const M Cp = M(2) * w1 * k22p + w2 * (be * k22p - ga * k12p);
        const M Cq = M(2) * w1 * k22c + w2 * (be * k22c - ga * k12c);
        const M t3 = e0e1 * rl * rl * rllp, t4 = e0e1 * rllp * rlp * rlp;
        const M pref = -k.G * M(0.5) * tri_area_of<M>(P, t);
        const V3<M> gl1 = rl * e0, glp2 = rlp * e1;
        const V3<M> gc0 = (t3 - rllp) * e0 + (t4 - rllp) * e1, gc1 = rllp * e1 - t3 * e0, gc2 = rllp * e0 - t4 * e1;
        sk(i0, pref * (M(-1) * (Cl * gl1 + Cp * glp2) + Cq * gc0));
        sk(i1, pref * (Cl * gl1 + Cq * gc1));
        sk(i2, pref * (Cp * glp2 + Cq * gc2));
        return;
    }
    const M l = norm3(e0), lp = norm3(e1);
    const M e0e1 = dot3(e0, e1);
    const M sin_phi = norm3(cross3(e0, e1)) / (l * lp);
    const M cos_phi = e0e1 / (l * lp);
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
    const M G = k.G, Cc = k.C;
    const M pref = -G / M(2) * tri_area_of<M>(P, t);
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
        sk(id[i], fv);
    }
}

// RBCParticle link term (WLC + POW), src/fsi/RBCParticle.hh:148-169 with
// RBCParameters::in_plane_ks_kp (RBCParticle.hh:27-44), m = 2, x0 = 1/2.2.
template <class M, class PS, class Sink>
__device__ void rbc_link(const ParticleDev& P, int l, const PS& ps, Sink& sk) {
    const double x0 = 1. / 2.2;
    const double ks_c1 = 0.25 * (6. * x0 + (3 * x0 * x0 - 2 * x0 * x0 * x0) / ((1 - x0) * (1 - x0)));
    const double ks_c2 = x0 / (2. * (1 - x0) * (1 - x0) * (1 - x0)) + 0.25 * (1. - 1. / ((1 - x0) * (1 - x0)));
    const double l0 = P.link_len[l];
    const double kp_c1 = -1. / (l0 * l0), kp_c2 = 3. / (l0 * l0);
    const double G_lhs = 4. * l0 * P.prm[BIB_P_SHEAR_MODULUS] / sqrt(3.0);
    const double den = ks_c1 * kp_c2 - ks_c2 * kp_c1;
    const M ks = (M)(-kp_c1 * G_lhs / den), kp = (M)(ks_c1 * G_lhs / den);
    const int a = P.links[2 * l], b = P.links[2 * l + 1];
    const V3<M> dv = ps(a) - ps(b);
    const M L = norm3(dv);
    const M x = L / (M)(l0 * 2.2);
    const M df = M(-0.25) * ks * (M(6) * x + (M(3) * x * x - M(2) * x * x * x) / ((M(1) - x) * (M(1) - x))) + kp / (L * L);
    const V3<M> fv = (df / L) * dv;
    sk(a, fv);
    sk(b, M(-1) * fv);
}

// RBCParticle triangle terms: global + local area and volume penalties,
// src/fsi/RBCParticle.hh:175-213 with tri::triangle_area_and_gradient and
// tri::grad_signed_volume (TriangleUtils.h:58-120).  The volume gradient is
// translation invariant on a closed surface, so it is taken relative to the centre.
template <class M, class PS, class Sink>
__device__ void rbc_triangle(const ParticleDev& P, int t, int4 ti, const PS& ps, const MemCoef<M>& k, Sink& sk) {
    const int i0 = ti.x, i1 = ti.y, i2 = ti.z;
    const V3<M> v0 = ps(i0), v1 = ps(i1), v2 = ps(i2);
    const M v01v11 = v0.y - v1.y, v02v22 = v0.z - v2.z, v02v12 = v0.z - v1.z;
    const M v01v21 = v0.y - v2.y, v00v20 = v0.x - v2.x, v00v10 = v0.x - v1.x;
    const M a = v01v11 * v02v22 - v02v12 * v01v21;
    const M b = v02v12 * v00v20 - v00v10 * v02v22;
    const M c = v00v10 * v01v21 - v01v11 * v00v20;
    const M la = M(0.5) * fast_sqrt(a * a + b * b + c * c);
    const M denom = fast_div(M(1), M(4) * la);
    const V3<M> g0 = mk3<M>((b * (v2.z - v1.z) + c * (v1.y - v2.y)) * denom, (a * (v1.z - v2.z) + c * (v2.x - v1.x)) * denom,
                            (a * (v2.y - v1.y) + b * (v1.x - v2.x)) * denom);
    const V3<M> g1 = mk3<M>((b * v02v22 + c * (v2.y - v0.y)) * denom, (a * (v2.z - v0.z) + c * v00v20) * denom,
                            (a * v01v21 + b * (v2.x - v0.x)) * denom);
    const V3<M> g2 = mk3<M>((b * (v1.z - v0.z) + c * v01v11) * denom, (a * v02v12 + c * (v1.x - v0.x)) * denom,
                            (a * (v1.y - v0.y) + b * v00v10) * denom);
    // the global penalty differences are evaluated once per particle, in FP64
    const M a0t = tri_area_of<M>(P, t);
    M df_area = k.df_area_global;
    df_area += fast_div(k.k_area_local * (a0t - la), a0t);
    sk(i0, df_area * g0);
    sk(i1, df_area * g1);
    sk(i2, df_area * g2);
    sk(i0, k.df_vol6 * cross3(v1, v2));
    sk(i1, k.df_vol6 * cross3(v2, v0));
    sk(i2, k.df_vol6 * cross3(v0, v1));
}

// Dihedral bending of one adjacent-triangle pair, src/fsi/RBCParticle.hh:217-246 with
// tri::grad_angle_between_pair (TriangleUtils.h:139-164).
template <class M, class PS, class Sink>
__device__ void rbc_pair(const ParticleDev& P, int p, const PS& ps, const MemCoef<M>& k, Sink& sk) {
    const int4 qq = __ldg(reinterpret_cast<const int4*>(P.pairs) + p);
    const int q[4] = {qq.x, qq.y, qq.z, qq.w};
    const V3<M> v0 = ps(q[0]), v1 = ps(q[1]), v2 = ps(q[2]), v3 = ps(q[3]);
    const V3<M> e0 = v1 - v0, e1 = v2 - v0, e2 = v3 - v0;
    const M e1n = norm3(e1);
    const V3<M> e1u = div3(e1, e1n);
    const V3<M> n1 = cross3(e0, e1), n2 = cross3(e1, e2);
    const M n1n = norm3(n1), n2n = norm3(n2);
    const V3<M> n1u = div3(n1, n1n), n2u = div3(n2, n2n);
    const M cos_t = dot3(n1u, n2u);
    const M sin_t = (dot3(n1 - n2, v1 - v3) > M(0) ? M(1) : M(-1)) * norm3(cross3(n1u, n2u));
    M c0, c1;
    if constexpr (sizeof(M) == sizeof(float)) {
        const float2 cs = __ldg(reinterpret_cast<const float2*>(P.pair_cs_f) + p);
        c0 = cs.x, c1 = cs.y;
    } else {
        c0 = pair_c<M>(P, p, 0), c1 = pair_c<M>(P, p, 1);
    }
    const M pref = k.kb * (-c0 * sin_t + c1 * cos_t);
    sk(q[0], pref * (fast_div(dot3(e1u, e1 - e2), n2n) * n2u + fast_div(dot3(e1u, e1 - e0), n1n) * n1u));
    sk(q[1], pref * (fast_div(-e1n, n1n) * n1u));
    sk(q[2], pref * (fast_div(dot3(e1u, e2), n2n) * n2u + fast_div(dot3(e1u, e0), n1n) * n1u));
    sk(q[3], pref * (fast_div(-e1n, n2n) * n2u));
}

// Forces on the three corners of one triangle, summed in registers and handed on once.
template <class M>
struct CornerSink {
    int id[3];
    V3<M> f[3];
    __device__ __forceinline__ void operator()(int v, V3<M> g) {
        if (v == id[0]) f[0] = f[0] + g;
        else if (v == id[1]) f[1] = f[1] + g;
        else f[2] = f[2] + g;
    }
};

// One CTA per particle: vertex forces at X_n (ParticleBase3D::reset_forces +
// compute_forces), accumulated in shared memory.
template <class M>
__device__ __forceinline__ void membrane_block(const ParticleDev& P, const IbView& V, unsigned char* smem_raw) {
    M* sf = reinterpret_cast<M*>(smem_raw);
    const double* __restrict__ pos = V.pos;
    double* __restrict__ force = V.force;
    const double* st = V.stats + STATS * P.lpid;
    const double area = st[0], volume = st[1];
    // gridDim.y CTAs share the elements of one particle: each sums its share in shared memory
    // and adds it to the force array (seeded by k_force_seed) with atomics
    const int split = gridDim.y;
    const int e0 = blockIdx.y * blockDim.x + threadIdx.x, es = split * blockDim.x;
    // the force decorators come first (ImmersedBoundaryDynamics_forces.hh:293-296)
    if (split == 1 && V.inter.nwall > 0) {
        for (int i = threadIdx.x; i < P.nv; i += blockDim.x) {
            double fw[3];
            wall_force(V.inter, pos + 3LL * (P.v0 + i), fw);
            sf[3 * i] = (M)fw[0];
            sf[3 * i + 1] = (M)fw[1];
            sf[3 * i + 2] = (M)fw[2];
        }
    } else {
        for (int i = threadIdx.x; i < 3 * P.nv; i += blockDim.x) sf[i] = M(0);
    }
    // FP64 element arithmetic uses absolute positions as the reference does; reduced
    // precision stages the positions relative to the centre of mass in shared memory
    // (exact FP64 subtraction, then rounding) so the element loops read them from there.
    const bool rel = sizeof(M) < sizeof(double);
    M* sp = sf + 3 * P.nv;
    if (rel) {
        const double* pp = pos + 3LL * P.v0;
        const double c[3] = {st[2], st[3], st[4]};
        for (int i = threadIdx.x; i < P.nv; i += blockDim.x) {
            sp[3 * i] = (M)(pp[3 * i] - c[0]);
            sp[3 * i + 1] = (M)(pp[3 * i + 1] - c[1]);
            sp[3 * i + 2] = (M)(pp[3 * i + 2] - c[2]);
        }
    }
    // the per-particle constants (FP64 divisions) once per CTA
    __shared__ MemCoef<M> kc;
    if (threadIdx.x == 0) kc = mem_coef<M>(P, area, volume);
    __syncthreads();
    AtomicSink<M> sk{sf};
    const int skalak = P.model != BIB_MODEL_CAPSULE_NEOHOOKEAN;
    const bool capsule = P.model == BIB_MODEL_CAPSULE_NEOHOOKEAN || P.model == BIB_MODEL_CAPSULE_SKALAK ||
                         P.model == BIB_MODEL_SKALAK_BENDING;
    const bool rbc_terms = P.model == BIB_MODEL_RBC_WLCPOW || P.model == BIB_MODEL_SKALAK_BENDING;
    const MemCoef<M> k = kc;
    auto run = [&](const auto& ps) {
        // triangle terms (capsule law and RBC area / volume penalties) of one triangle are
        // summed per corner before they reach the shared accumulators
        if (capsule || rbc_terms)
            for (int t = e0; t < P.nt; t += es) {
                const V3<M> z = mk3<M>(0, 0, 0);
                const int4 ti = __ldg(reinterpret_cast<const int4*>(P.tri4) + t);
                CornerSink<M> cs{{ti.x, ti.y, ti.z}, {z, z, z}};
                if (capsule) capsule_triangle<M>(P, t, ti, ps, skalak, k, cs);
                if (rbc_terms) rbc_triangle<M>(P, t, ti, ps, k, cs);
                for (int c = 0; c < 3; ++c) sk(cs.id[c], cs.f[c]);
            }
        if (P.model == BIB_MODEL_RBC_WLCPOW)
            for (int l = e0; l < P.nl; l += es) rbc_link<M>(P, l, ps, sk);
        if (rbc_terms)
            for (int p = e0; p < P.np; p += es) rbc_pair<M>(P, p, ps, k, sk);
    };
    if (rel) run(SharedPos<M>{sp});
    else run(GlobalPos<M>{pos + 3LL * P.v0, {0.0, 0.0, 0.0}});
    __syncthreads();
    if (split == 1) {
        for (int i = threadIdx.x; i < 3 * P.nv; i += blockDim.x) force[3LL * P.v0 + i] = (double)sf[i];
    } else {
        for (int i = threadIdx.x; i < 3 * P.nv; i += blockDim.x)
            if (sf[i] != M(0)) atomicAdd(force + 3LL * P.v0 + i, (double)sf[i]);
    }
}

// The vertex forces before a split membrane launch adds into them: the wall-interaction
// decorators, or zero.
__global__ void __launch_bounds__(128) k_force_seed(IbView V) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V.nvert) return;
    double fw[3] = {0.0, 0.0, 0.0};
    if (V.inter.nwall > 0) wall_force(V.inter, V.pos + 3LL * v, fw);
    V.force[3LL * v] = fw[0];
    V.force[3LL * v + 1] = fw[1];
    V.force[3LL * v + 2] = fw[2];
}

template <class M, bool BATCH>
__global__ void __launch_bounds__(512) k_membrane(const ParticleDev* __restrict__ parts, IbView v1,
                                                   const IbView* __restrict__ views) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const ParticleDev& P = parts[blockIdx.x];
    membrane_block<M>(P, BATCH ? views[P.inst] : v1, smem_raw);
}

// Deterministic membrane forces: one thread per vertex sums the contributions of its
// incident links, triangles and adjacent-triangle pairs, visited in the order of the
// reference's element loops (RBCParticle.hh:148-246: links, then triangles with the area
// term before the volume term, then pairs).  Each incident element is evaluated once per
// corner, so the element arithmetic is repeated 2-4 times; no atomics, bit-reproducible.
// The Skalak + bending composite sums the capsule part and the RBC part separately, as
// the reference does when both particle classes act on the same vertices.
constexpr int INC_LINK = 0, INC_TRI = 1, INC_PAIR = 2;

template <class M>
__global__ void __launch_bounds__(128) k_membrane_gather(int nvert, const int* __restrict__ vert_particle,
                                                          const ParticleDev* __restrict__ parts,
                                                          const double* __restrict__ pos, double* __restrict__ force,
                                                          const double* __restrict__ stats, Interactions inter) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nvert) return;
    const int pid = vert_particle[g];
    const ParticleDev& P = parts[pid];
    const int lv = g - P.v0;
    const double* st = stats + STATS * pid;
    const double area = st[0], volume = st[1];
    const bool rel = sizeof(M) < sizeof(double);
    const GlobalPos<M> ps{pos + 3LL * P.v0, {rel ? st[2] : 0.0, rel ? st[3] : 0.0, rel ? st[4] : 0.0}};
    const bool capsule = P.model == BIB_MODEL_CAPSULE_NEOHOOKEAN || P.model == BIB_MODEL_CAPSULE_SKALAK ||
                         P.model == BIB_MODEL_SKALAK_BENDING;
    const bool rbc_terms = P.model == BIB_MODEL_RBC_WLCPOW || P.model == BIB_MODEL_SKALAK_BENDING;
    const int skalak = P.model != BIB_MODEL_CAPSULE_NEOHOOKEAN;
    const MemCoef<M> k = mem_coef<M>(P, area, volume);
    GatherSink<M> cap{lv, mk3<M>(0, 0, 0)}, rbc{lv, mk3<M>(0, 0, 0)};
    for (int e = P.inc_off[lv]; e < P.inc_off[lv + 1]; ++e) {
        const int code = P.inc[e];
        const int type = code >> 29, id = code & ((1 << 29) - 1);
        if (type == INC_LINK) {
            if (P.model == BIB_MODEL_RBC_WLCPOW) rbc_link<M>(P, id, ps, rbc);
        } else if (type == INC_TRI) {
            const int4 ti = __ldg(reinterpret_cast<const int4*>(P.tri4) + id);
            if (capsule) capsule_triangle<M>(P, id, ti, ps, skalak, k, cap);
            if (rbc_terms) rbc_triangle<M>(P, id, ti, ps, k, rbc);
        } else if (type == INC_PAIR && rbc_terms) {
            rbc_pair<M>(P, id, ps, k, rbc);
        }
    }
    V3<M> f = P.model == BIB_MODEL_SKALAK_BENDING ? cap.acc + rbc.acc : (capsule ? cap.acc : rbc.acc);
    double fw[3] = {0.0, 0.0, 0.0};
    if (inter.nwall > 0) wall_force(inter, pos + 3LL * g, fw);
    force[3LL * g] = fw[0] + (double)f.x;
    force[3LL * g + 1] = fw[1] + (double)f.y;
    force[3LL * g + 2] = fw[2] + (double)f.z;
}

// One CTA per particle: area, signed volume and area-weighted centroid of X_{n+1}
// (DeformableParticle3D::update, DeformableParticle3D.hh:54-82), then the periodic
// centre-of-mass remap (ParticleBase3D::map_center_of_mass_to_periodic_grid,
// ParticleBase.hh:111-136).  M = double follows the reference with absolute positions.
// M = float (reduced-precision lattices) evaluates each triangle in FP32 on positions
// relative to the previous centre of mass (exact FP64 subtraction, then rounding) and
// accumulates in FP64; the signed volume of the closed surface does not depend on the
// origin.
// Sums of five per-thread values over the block into out[0..4] (shared): the partials go
// to red (5 x blockDim.x doubles), then one warp per quantity adds them up.
__device__ __forceinline__ void block_sum5(const double v[5], double* red, double* out) {
    const int n = blockDim.x, t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < 5; ++k) red[k * n + t] = v[k];
    __syncthreads();
    const int lane = t & 31, nw = n >> 5;
    for (int q = t >> 5; q < 5; q += nw) {
        double s = 0.0;
        for (int i = lane; i < n; i += 32) s += red[q * n + i];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) out[q] = s;
    }
    __syncthreads();
}

// Per-triangle area, signed volume and area-weighted centroid of X_{n+1}, summed over the
// triangles e0, e0 + es, ... by this CTA into sum[0..4] (shared; valid for every thread).
template <class M>
__device__ __forceinline__ void update_sums(const ParticleDev& P, const IbView& V, float* sp, double* red, double* sum,
                                            int e0, int es) {
    const double* pv = V.pos_next + 3LL * P.v0;
    const double* st = V.stats + STATS * P.lpid;
    const bool rel = sizeof(M) < sizeof(double);
    const double c0 = rel ? st[2] : 0.0, c1 = rel ? st[3] : 0.0, c2 = rel ? st[4] : 0.0;
    if (rel) {  // one FP64 subtraction and rounding per vertex coordinate
        for (int i = threadIdx.x; i < P.nv; i += blockDim.x) {
            sp[3 * i] = (float)(pv[3 * i] - c0);
            sp[3 * i + 1] = (float)(pv[3 * i + 1] - c1);
            sp[3 * i + 2] = (float)(pv[3 * i + 2] - c2);
        }
        __syncthreads();
    }
    auto vert = [&](int i) {
        return rel ? mk3<M>((M)sp[3 * i], (M)sp[3 * i + 1], (M)sp[3 * i + 2])
                   : mk3<M>((M)(pv[3 * i] - c0), (M)(pv[3 * i + 1] - c1), (M)(pv[3 * i + 2] - c2));
    };
    // per-thread partial sums in M (a few triangles each), block sums in FP64
    M ta = 0, tv = 0, tcx = 0, tcy = 0, tcz = 0;
    for (int t = e0; t < P.nt; t += es) {
        const int4 ti = __ldg(reinterpret_cast<const int4*>(P.tri4) + t);
        const V3<M> A = vert(ti.x), B = vert(ti.y), Cv = vert(ti.z);
        const M dA = norm3(cross3(B - A, Cv - A)) * M(0.5);
        ta += dA;
        // multiplications by 1/6 and 1/3 instead of the reference's divisions (FP64 division
        // is a long instruction sequence on this part); differences are within one ulp per term
        tv += dot3(A, cross3(B, Cv)) * (M(1) / M(6));
        const V3<M> cen = (M(1) / M(3)) * (A + B + Cv);
        tcx += cen.x * dA;
        tcy += cen.y * dA;
        tcz += cen.z * dA;
    }
    const double part[5] = {(double)ta, (double)tv, (double)tcx, (double)tcy, (double)tcz};
    block_sum5(part, red, sum);
}

// A, V and the centre from the sums (relative to the previous centre for M = float), the
// periodic centre-of-mass remap, and the shift of the vertices by whole periods.
template <class M>
__device__ __forceinline__ void update_finish(const ParticleDev& P, const IbView& V, const double* sum, double* delta) {
    const LatticeDesc& d = V.d;
    double* pos_next = V.pos_next;
    double* st = V.stats + STATS * P.lpid;
    if (threadIdx.x == 0) {
        const bool rel = sizeof(M) < sizeof(double);
        const double c0 = rel ? st[2] : 0.0, c1 = rel ? st[3] : 0.0, c2 = rel ? st[4] : 0.0;
        const double sa = sum[0], sv = sum[1];
        const double com[3] = {c0 + sum[2] / sa, c1 + sum[3] / sa, c2 + sum[4] / sa};
        const int N[3] = {d.nx, d.ny, d.nz};
        const int per[3] = {d.px, d.py, d.pz};
        double np_[3];
        for (int a = 0; a < 3; ++a) {
            np_[a] = com[a];
            if (per[a]) np_[a] = com[a] - (double)N[a] * floor((com[a] - (-0.5)) * d.inv_n[a]);
            delta[a] = np_[a] - com[a];
        }
        st[0] = sa;
        st[1] = sv;
        st[2] = np_[0];
        st[3] = np_[1];
        st[4] = np_[2];
    }
    __syncthreads();
    if (delta[0] != 0.0 || delta[1] != 0.0 || delta[2] != 0.0) {
        for (int i = threadIdx.x; i < P.nv; i += blockDim.x) {
            const int64_t g = 3LL * (P.v0 + i);
            pos_next[g] += delta[0];
            pos_next[g + 1] += delta[1];
            pos_next[g + 2] += delta[2];
        }
    }
}

template <class M>
__device__ __forceinline__ void update_block(const ParticleDev& P, const IbView& V, float* sp, double* red,
                                             double* delta) {
    __shared__ double sum[5];
    update_sums<M>(P, V, sp, red, sum, threadIdx.x, blockDim.x);
    update_finish<M>(P, V, sum, delta);
}

// Few particles: gridDim.y CTAs per particle write partial sums, one CTA per particle adds
// them in slice order and finishes the update.
constexpr int kMaxUpdateSplit = 64;

template <class M>
__global__ void __launch_bounds__(256) k_update_partial(const ParticleDev* __restrict__ parts, IbView v1,
                                                         double* __restrict__ partial) {
    __shared__ double red[5 * 256];
    __shared__ double sum[5];
    extern __shared__ __align__(16) float sp[];
    const ParticleDev& P = parts[blockIdx.x];
    update_sums<M>(P, v1, sp, red, sum, blockIdx.y * blockDim.x + threadIdx.x, gridDim.y * blockDim.x);
    if (threadIdx.x < 5) partial[(blockIdx.x * (size_t)gridDim.y + blockIdx.y) * 5 + threadIdx.x] = sum[threadIdx.x];
}

template <class M>
__global__ void __launch_bounds__(256) k_update_finish(const ParticleDev* __restrict__ parts, IbView v1,
                                                        const double* __restrict__ partial, int split) {
    __shared__ double sum[5];
    __shared__ double delta[3];
    const ParticleDev& P = parts[blockIdx.x];
    if (threadIdx.x < 5) {
        double a = 0.0;
        for (int y = 0; y < split; ++y) a += partial[(blockIdx.x * (size_t)split + y) * 5 + threadIdx.x];
        sum[threadIdx.x] = a;
    }
    __syncthreads();
    update_finish<M>(P, v1, sum, delta);
}

template <class M, bool BATCH>
__global__ void __launch_bounds__(256) k_particle_update(const ParticleDev* __restrict__ parts, IbView v1,
                                                          const IbView* __restrict__ views) {
    __shared__ double red[5 * 256];
    __shared__ double delta[3];
    extern __shared__ __align__(16) float sp[];  // M = float: relative vertex positions
    const ParticleDev& P = parts[blockIdx.x];
    update_block<M>(P, BATCH ? views[P.inst] : v1, sp, red, delta);
}

// ---------------------------------------------------------------- voxelization
// RayTracer::tri_ray_intersect (fsi/RayTracer.hh:80-108) for the ray from (px, py, 0) along
// +z, in the reference's operation order and without fused multiply-adds, so the
// intersection heights (and therefore the phase field) are the reference's to the bit.
__device__ __forceinline__ double dot_nofma(const double* a, const double* b) {
    double r = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) r = __dadd_rn(r, __dmul_rn(a[d], b[d]));
    return r;
}
__device__ __forceinline__ void cross_nofma(const double* a, const double* b, double* c) {
    c[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1]));
    c[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2]));
    c[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]));
}
__device__ __forceinline__ bool tri_ray_z(const double* v0, const double* v1, const double* v2, double px, double py,
                                          double& dist) {
    const double e1[3] = {__dsub_rn(v1[0], v0[0]), __dsub_rn(v1[1], v0[1]), __dsub_rn(v1[2], v0[2])};
    const double e2[3] = {__dsub_rn(v2[0], v0[0]), __dsub_rn(v2[1], v0[1]), __dsub_rn(v2[2], v0[2])};
    const double dir[3] = {0.0, 0.0, 1.0};
    double q[3];
    cross_nofma(dir, e2, q);
    const double a = dot_nofma(e1, q);
    if (fabs(a) < DBL_EPSILON) return false;
    const double f = __drcp_rn(a);
    const double sv[3] = {__dsub_rn(px, v0[0]), __dsub_rn(py, v0[1]), __dsub_rn(0.0, v0[2])};
    const double u = __dmul_rn(f, dot_nofma(sv, q));
    if (u < 0.0) return false;
    double r[3];
    cross_nofma(sv, e1, r);
    const double v = __dmul_rn(f, dot_nofma(dir, r));
    if (v < 0.0 || __dadd_rn(u, v) > 1.0) return false;
    dist = __dmul_rn(f, dot_nofma(e2, r));
    return true;
}

// One CTA per particle, one thread per triangle: z-rays through the integer (x, y) points of
// the triangle's xy box (RayTracer::find_intersections_z, RayTracer.hh:18-40); each hit goes
// to its (periodically wrapped) column, height wrapped into [-1/2, nz - 1/2) (ZBuffer::put,
// Arithmetic1D::remap_pos).  Columns are numbered x fastest.
__global__ void __launch_bounds__(128) k_voxel_rays(LatticeDesc d, const ParticleDev* __restrict__ parts,
                                                     const double* __restrict__ pos, int* __restrict__ count,
                                                     double* __restrict__ zbuf, int cap, int* __restrict__ overflow) {
    const ParticleDev& P = parts[blockIdx.x];
    const double* pv = pos + 3LL * P.v0;
    const int64_t ncol = (int64_t)d.nx * d.ny;
    for (int t = threadIdx.x; t < P.nt; t += blockDim.x) {
        const double* v0 = pv + 3 * P.tri[3 * t];
        const double* v1 = pv + 3 * P.tri[3 * t + 1];
        const double* v2 = pv + 3 * P.tri[3 * t + 2];
        double x0 = fmin(v0[0], fmin(v1[0], v2[0])), x1 = fmax(v0[0], fmax(v1[0], v2[0]));
        double y0 = fmin(v0[1], fmin(v1[1], v2[1])), y1 = fmax(v0[1], fmax(v1[1], v2[1]));
        // a triangle wider than the lattice (or not finite) only arises from a diverged
        // membrane: flag it instead of casting rays through a runaway box
        if (!(x1 - x0 < (double)d.nx && y1 - y0 < (double)d.ny)) {
            atomicExch(overflow, 1);
            continue;
        }
        if (!d.px) x0 = fmax(x0, -1.0), x1 = fmin(x1, (double)d.nx);  // rays outside a walled axis are dropped
        if (!d.py) y0 = fmax(y0, -1.0), y1 = fmin(y1, (double)d.ny);
        const int64_t i0 = (int64_t)ceil(x0), i1 = (int64_t)floor(x1);
        const int64_t j0 = (int64_t)ceil(y0), j1 = (int64_t)floor(y1);
        for (int64_t i = i0; i <= i1; ++i)
            for (int64_t j = j0; j <= j1; ++j) {
                double z;
                if (!tri_ray_z(v0, v1, v2, (double)i, (double)j, z)) continue;
                int64_t cx = i, cy = j;
                if (d.px) cx = pmod(cx, d.nx);
                else if (cx < 0 || cx >= d.nx) continue;
                if (d.py) cy = pmod(cy, d.ny);
                else if (cy < 0 || cy >= d.ny) continue;
                if (d.pz) z = __dsub_rn(z, __dmul_rn((double)d.nz, floor(__dmul_rn(__dsub_rn(z, -0.5), d.inv_n[2]))));
                const int64_t c = cx + (int64_t)d.nx * cy;
                const int slot = atomicAdd(count + c, 1);
                if (slot < cap) zbuf[slot * ncol + c] = z;
                else atomicExch(overflow, 1);
            }
    }
}

// One thread per column: sort its heights and fill the column from below by parity
// (apply_voxelization, ImmersedBoundaryDynamics_voxelization.hh:121-161); resets the count.
// Heights of column c sit at zbuf[slot * ncol + c], so a warp reads slot e of 32 columns at once.
__global__ void __launch_bounds__(128) k_voxel_fill(LatticeDesc d, int* __restrict__ count, double* __restrict__ zbuf,
                                                     int cap, uint8_t* __restrict__ phase) {
    const int64_t ncol = (int64_t)d.nx * d.ny;
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const int m = min(count[c], cap);
    count[c] = 0;
    double* zl = zbuf + c;
    for (int e = 1; e < m; ++e) {  // insertion sort, ascending, in place
        const double z = zl[e * ncol];
        int p = e;
        while (p > 0 && zl[(p - 1) * ncol] > z) {
            zl[p * ncol] = zl[(p - 1) * ncol];
            --p;
        }
        zl[p * ncol] = z;
    }
    const int64_t plane = ncol;
    uint8_t inside = 0;
    double z_last = -10000.0;
    for (int e = 0; e <= m; ++e) {
        const double ze = e < m ? zl[e * ncol] : 0.0;
        int64_t lo, hi;
        if (e < m) {
            lo = max((int64_t)ceil(z_last), (int64_t)0);
            hi = min((int64_t)floor(ze), (int64_t)d.nz - 1);
        } else {
            if (!(ceil(z_last) < (double)(d.nz - 1))) break;
            lo = max((int64_t)ceil(z_last), (int64_t)0);
            hi = d.nz - 1;
        }
        for (int64_t z = lo; z <= hi; ++z) phase[c + plane * z] = inside;
        if (e < m) {
            z_last = ze;
            inside ^= 1;
        }
    }
}

// ---------------------------------------------------------------- particle-particle interactions
// Pair search on a hashed cell list: cells of at least the largest cutoff, each vertex keyed
// by the hash of its cell, vertices sorted by key (stable: vertex order within a bucket).
struct PairCells {
    int nc[3];
    double cs[3];
    unsigned mask;
};

__device__ __forceinline__ int pair_cell(const LatticeDesc& d, const PairCells& g, int a, double x) {
    const int N = a == 0 ? d.nx : (a == 1 ? d.ny : d.nz);
    const int per = a == 0 ? d.px : (a == 1 ? d.py : d.pz);
    if (per) x -= (double)N * floor(x * d.inv_n[a]);
    int c = (int)floor(x / g.cs[a]);
    return c < 0 ? 0 : (c >= g.nc[a] ? g.nc[a] - 1 : c);
}
__device__ __forceinline__ unsigned cell_hash(const PairCells& g, int cx, int cy, int cz) {
    return ((unsigned)cx * 73856093u ^ (unsigned)cy * 19349663u ^ (unsigned)cz * 83492791u) & g.mask;
}

// the buckets of the previous step's sort go back to empty
__global__ void __launch_bounds__(128) k_pp_clear(int nvert, const uint32_t* __restrict__ prev_keys, int* start,
                                                   int* end) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nvert) return;
    start[prev_keys[s]] = 0;
    end[prev_keys[s]] = 0;
}

__global__ void __launch_bounds__(128) k_pp_keys(LatticeDesc d, PairCells g, int nvert, const double* __restrict__ pos,
                                                  uint32_t* __restrict__ keys, uint32_t* __restrict__ ids) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvert) return;
    const double* p = pos + 3LL * v;
    keys[v] = cell_hash(g, pair_cell(d, g, 0, p[0]), pair_cell(d, g, 1, p[1]), pair_cell(d, g, 2, p[2]));
    ids[v] = (uint32_t)v;
}

__global__ void __launch_bounds__(128) k_pp_bounds(int nvert, const uint32_t* __restrict__ keys, int* start, int* end) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nvert) return;
    const uint32_t k = keys[s];
    if (s == 0 || keys[s - 1] != k) start[k] = s;
    if (s == nvert - 1 || keys[s + 1] != k) end[k] = s + 1;
}

// Arithmetic1D::min_mod_diff (Periodicity.h:27-35, 96-99) on periodic axes
__device__ __forceinline__ double min_image(const LatticeDesc& d, int a, double dx) {
    const int per = a == 0 ? d.px : (a == 1 ? d.py : d.pz);
    if (!per) return dx;
    const double N = (double)(a == 0 ? d.nx : (a == 1 ? d.ny : d.nz));
    return dx - floor(dx * d.inv_n[a] + 0.5) * N;
}

// One thread per vertex: the sum over partners j of other particles within the cutoff of
// (-phi(d) / d) (x_j - x_i) (CollisionHandler::handle_collision, CollisionForces.h:187-199),
// added to the vertex's force.  Every pair is evaluated from both ends, so no atomics.
__global__ void __launch_bounds__(128) k_pp_forces(LatticeDesc d, Interactions I, PairCells g, int nvert,
                                                    const double* __restrict__ pos, const int* __restrict__ owner,
                                                    const uint32_t* __restrict__ ids, const int* __restrict__ start,
                                                    const int* __restrict__ end, double* __restrict__ force) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nvert) return;
    const double xi[3] = {pos[3LL * i], pos[3LL * i + 1], pos[3LL * i + 2]};
    if (!(isfinite(xi[0]) && isfinite(xi[1]) && isfinite(xi[2]))) return;
    const int oi = owner[i];
    const int c[3] = {pair_cell(d, g, 0, xi[0]), pair_cell(d, g, 1, xi[1]), pair_cell(d, g, 2, xi[2])};
    const int per[3] = {d.px, d.py, d.pz};
    const double cut2 = I.pp_cut * I.pp_cut;
    double f[3] = {0.0, 0.0, 0.0};
    unsigned seen[27];
    int nseen = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int n[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
                bool ok = true;
                for (int a = 0; a < 3; ++a) {
                    if (n[a] < 0 || n[a] >= g.nc[a]) {
                        if (!per[a]) ok = false;
                        else n[a] = (n[a] + g.nc[a]) % g.nc[a];
                    }
                }
                if (!ok) continue;
                const unsigned h = cell_hash(g, n[0], n[1], n[2]);
                bool dup = false;  // neighbour cells that share a bucket are visited once
                for (int q = 0; q < nseen; ++q) dup = dup || seen[q] == h;
                if (dup) continue;
                seen[nseen++] = h;
                for (int s = start[h]; s < end[h]; ++s) {
                    const int j = (int)ids[s];
                    if (owner[j] == oi) continue;
                    const double dr[3] = {min_image(d, 0, pos[3LL * j] - xi[0]), min_image(d, 1, pos[3LL * j + 1] - xi[1]),
                                          min_image(d, 2, pos[3LL * j + 2] - xi[2])};
                    const double dsq = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
                    if (!(dsq <= cut2)) continue;
                    const double dist = sqrt(dsq);
                    for (int k = 0; k < I.npp; ++k) {
                        if (!(dsq <= I.pp[k].r0 * I.pp[k].r0)) continue;
                        const double sc = -potential_eval(I.pp[k], dist) / dist;
                        f[0] += sc * dr[0];
                        f[1] += sc * dr[1];
                        f[2] += sc * dr[2];
                    }
                }
            }
    force[3LL * i] += f[0];
    force[3LL * i + 1] += f[1];
    force[3LL * i + 2] += f[2];
}

}  // namespace

size_t membrane_smem_bytes(int max_nv) { return (size_t)3 * max_nv * sizeof(double); }

size_t spread_sort_temp_bytes(int64_t nentries) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs((void*)nullptr, bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, (int)nentries, 0, 32);  // upper bound over the key widths
    return bytes;
}

int spread_key_bits(int64_t n) { return key_bits(n); }

size_t spread_sort_temp_bytes_pingpong(int64_t nentries, int end_bit) {
    size_t bytes = 0;
    cub::DoubleBuffer<uint32_t> k(nullptr, nullptr), v(nullptr, nullptr);
    if (cub::DeviceRadixSort::SortPairs(nullptr, bytes, k, v, (int)nentries, 0, end_bit) != cudaSuccess) return SIZE_MAX;
    return bytes;
}

cudaError_t launch_spread_sorted(const LatticeDesc& d, const IbDesc& ib, bool f64_field, int nvert, const double* pos,
                                 const double* force, void* field, uint32_t* keys0, uint32_t* keys1, uint32_t* ids0,
                                 uint32_t* ids1, void* temp, size_t temp_bytes, cudaStream_t s) {
    const int sup = ib.dirac == BIB_DIRAC_PESKIN ? 4 : 3;
    const int64_t ne = (int64_t)nvert * sup * sup * sup;
    k_spread_keys<<<(nvert + 127) / 128, 128, 0, s>>>(d, ib, nvert, pos, keys0, ids0, nullptr);
    cub::DoubleBuffer<uint32_t> k(keys0, keys1), v(ids0, ids1);
    size_t tb = temp_bytes;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(temp, tb, k, v, (int)ne, 0, key_bits(d.n), s);
    if (e != cudaSuccess) return e;
    const unsigned ge = (unsigned)((ne + 127) / 128);
    if (f64_field)
        k_spread_reduce<double><<<ge, 128, 0, s>>>(d, ib, ne, k.Current(), v.Current(), pos, force, (double*)field);
    else
        k_spread_reduce<float><<<ge, 128, 0, s>>>(d, ib, ne, k.Current(), v.Current(), pos, force, (float*)field);
    return cudaGetLastError();
}

void configure_membrane_kernel(size_t smem) {
    // the limit is per kernel function: only ever raise it, other lattices may need more
    static size_t configured = 0;
    if (smem <= configured) return;
    configured = smem;
    cudaFuncSetAttribute(k_membrane<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_membrane<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_membrane<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_membrane<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // 3 floats per vertex, at most half of the membrane kernel's 3 doubles per vertex
    cudaFuncSetAttribute(k_particle_update<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(smem / 2));
    cudaFuncSetAttribute(k_particle_update<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(smem / 2));
    cudaFuncSetAttribute(k_update_partial<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(smem / 2));
}

IbView single_view(const Lattice& L, int fbuf) {
    IbView v{};
    v.d = L.d;
    v.ib = L.ib;
    v.pos = L.pos[L.pcur];
    v.pos_next = L.pos[1 - L.pcur];
    v.u = L.u;
    v.vel = L.vel;
    v.force = L.force;
    v.F = fbuf >= 0 ? L.F[fbuf] : nullptr;
    v.stats = L.stats;
    v.vbase = 0;
    v.nvert = L.nvert;
    v.inter = L.inter;
    v.order = L.visit_order;
    return v;
}

namespace {

template <bool BATCH>
void interpolate_any(int storage, int dirac, const IbView& v1, const IbView* views, const int* vinst, int nvert,
                     cudaStream_t s) {
    const unsigned g = (nvert + 127) / 128;
    const bool peskin = dirac == BIB_DIRAC_PESKIN;
    if (storage == BIB_STORAGE_F64) {
        if (peskin) k_interpolate_move<double, 4, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
        else k_interpolate_move<double, 3, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
    } else if (storage == BIB_STORAGE_F32) {
        if (peskin) k_interpolate_move<float, 4, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
        else k_interpolate_move<float, 3, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
    } else {
        if (peskin) k_interpolate_move<__half, 4, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
        else k_interpolate_move<__half, 3, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
    }
}

template <bool BATCH>
void spread_any(int storage, int dirac, const IbView& v1, const IbView* views, const int* vinst, int nvert,
                cudaStream_t s) {
    const unsigned g = (nvert + 127) / 128;
    const bool peskin = dirac == BIB_DIRAC_PESKIN;
    if (storage == BIB_STORAGE_F64) {
        if (peskin) k_spread<double, 4, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
        else k_spread<double, 3, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
    } else {
        if (peskin) k_spread<float, 4, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
        else if (!BATCH) k_spread_pairs<<<(unsigned)((2LL * nvert + 127) / 128), 128, 0, s>>>(v1, nvert);
        else k_spread<float, 3, BATCH><<<g, 128, 0, s>>>(v1, views, vinst, nvert);
    }
}

template <bool BATCH>
void membrane_any(int storage, const ParticleDev* parts, int np, const IbView& v1, const IbView* views, size_t smem,
                  int block, cudaStream_t s) {
    if (storage == BIB_STORAGE_F64) k_membrane<double, BATCH><<<np, block, smem, s>>>(parts, v1, views);
    else k_membrane<float, BATCH><<<np, block, smem, s>>>(parts, v1, views);
}

template <bool BATCH>
void update_any(int storage, const ParticleDev* parts, int np, const IbView& v1, const IbView* views, int max_nv,
                cudaStream_t s) {
    if (storage == BIB_STORAGE_F64) k_particle_update<double, BATCH><<<np, 256, 0, s>>>(parts, v1, views);
    else k_particle_update<float, BATCH><<<np, 256, 3 * sizeof(float) * max_nv, s>>>(parts, v1, views);
}

}  // namespace

void launch_interpolate_move(const Lattice& L, cudaStream_t s, int fold) {
    if (L.nvert == 0) return;
    if (fold < 0 || L.storage == BIB_STORAGE_F64) {
        interpolate_any<false>(L.storage, L.ib.dirac, single_view(L, -1), nullptr, nullptr, L.nvert, s);
        return;
    }
    IbView v = single_view(L, -1);
    v.Fold = L.F[fold];
    const unsigned g = (L.nvert + 127) / 128;
    const bool peskin = L.ib.dirac == BIB_DIRAC_PESKIN;
    if (L.storage == BIB_STORAGE_F32) {
        if (peskin) k_interpolate_move<float, 4, false, true><<<g, 128, 0, s>>>(v, nullptr, nullptr, L.nvert);
        else k_interpolate_move<float, 3, false, true><<<g, 128, 0, s>>>(v, nullptr, nullptr, L.nvert);
    } else {
        if (peskin) k_interpolate_move<__half, 4, false, true><<<g, 128, 0, s>>>(v, nullptr, nullptr, L.nvert);
        else k_interpolate_move<__half, 3, false, true><<<g, 128, 0, s>>>(v, nullptr, nullptr, L.nvert);
    }
}

void launch_force_clear(const Lattice& L, int fbuf, cudaStream_t s) {
    if (L.nvert == 0 || L.storage == BIB_STORAGE_F64) return;
    const int sup = L.ib.dirac == BIB_DIRAC_PESKIN ? 4 : 3;
    const int64_t threads = (int64_t)L.nvert * sup * sup;
    const unsigned g = (unsigned)((threads + 127) / 128);
    if (sup == 4) k_force_clear<4><<<g, 128, 0, s>>>(L.d, L.ib, L.nvert, L.spread_lo[fbuf], (float*)L.F[fbuf]);
    else k_force_clear<3><<<g, 128, 0, s>>>(L.d, L.ib, L.nvert, L.spread_lo[fbuf], (float*)L.F[fbuf]);
}

// CTAs per particle of the membrane kernel: enough to give every SM two CTAs, but at least
// one element per thread
int membrane_split(int np, int max_elems, int block) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    if (np <= 0 || np >= sms) return 1;
    const int want = (2 * sms + np - 1) / np;
    const int most = std::max(1, (max_elems + block - 1) / block);
    return std::max(1, std::min(want, most));
}

void launch_membrane_forces(const Lattice& L, cudaStream_t s) {
    const int np = (int)L.parts.size();
    if (np == 0) return;
    if (L.ib.spread_mode == BIB_SPREAD_DETERMINISTIC) {
        const unsigned g = (L.nvert + 127) / 128;
        if (L.storage == BIB_STORAGE_F64)
            k_membrane_gather<double><<<g, 128, 0, s>>>(L.nvert, L.vert_particle, L.pdev, L.pos[L.pcur], L.force, L.stats, L.inter);
        else
            k_membrane_gather<float><<<g, 128, 0, s>>>(L.nvert, L.vert_particle, L.pdev, L.pos[L.pcur], L.force, L.stats, L.inter);
        return;
    }
    // few particles: spread each particle's elements over several CTAs so the launch fills the GPU
    const int split = membrane_split(np, L.max_elems, L.membrane_block);
    if (split > 1) {
        const IbView v = single_view(L, -1);
        k_force_seed<<<(L.nvert + 127) / 128, 128, 0, s>>>(v);
        const dim3 grid((unsigned)np, (unsigned)split);
        if (L.storage == BIB_STORAGE_F64) k_membrane<double, false><<<grid, L.membrane_block, L.membrane_smem, s>>>(L.pdev, v, nullptr);
        else k_membrane<float, false><<<grid, L.membrane_block, L.membrane_smem, s>>>(L.pdev, v, nullptr);
        return;
    }
    membrane_any<false>(L.storage, L.pdev, np, single_view(L, -1), nullptr, L.membrane_smem, L.membrane_block, s);
}

size_t pp_sort_temp_bytes(int nvert, int bits) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs((void*)nullptr, bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, nvert, 0, bits);
    return bytes;
}

void launch_pp_forces(const Lattice& L, cudaStream_t s) {
    if (L.inter.npp == 0 || L.nvert == 0) return;
    if (L.inter.pp_search == BIB_PAIR_SEARCH_GRID) {
        // one CollisionHandler per potential, in order (ImmersedBoundaryDynamics_forces.hh:299-301)
        if (!L.rgrid.start) return;
        const int64_t box[6] = {0, L.d.nx - 1, 0, L.d.ny - 1, 0, L.d.nz - 1};
        const int per[3] = {L.d.px, L.d.py, L.d.pz};
        for (int k = 0; k < L.inter.npp; ++k)
            launch_ref_grid_forces(ref_grid(box, per, L.inter.pp[k].r0, L.nvert), L.rgrid, L.inter.pp[k],
                                   L.pos[L.pcur], L.vert_particle, L.force, false, nullptr, s);
        return;
    }
    if (!L.pgrid.table) return;
    const PairGrid& G = L.pgrid;
    PairCells g;
    for (int a = 0; a < 3; ++a) {
        g.nc[a] = G.nc[a];
        g.cs[a] = G.cs[a];
    }
    g.mask = G.table - 1;
    const unsigned b = (L.nvert + 127) / 128;
    k_pp_clear<<<b, 128, 0, s>>>(L.nvert, G.keys[1], G.start, G.end);
    k_pp_keys<<<b, 128, 0, s>>>(L.d, g, L.nvert, L.pos[L.pcur], G.keys[0], G.ids[0]);
    size_t tb = G.temp_bytes;
    cub::DeviceRadixSort::SortPairs(G.temp, tb, G.keys[0], G.keys[1], G.ids[0], G.ids[1], L.nvert, 0, G.bits, s);
    k_pp_bounds<<<b, 128, 0, s>>>(L.nvert, G.keys[1], G.start, G.end);
    k_pp_forces<<<b, 128, 0, s>>>(L.d, L.inter, g, L.nvert, L.pos[L.pcur], L.vert_particle, G.ids[1], G.start, G.end,
                                  L.force);
}

void launch_particle_update(const Lattice& L, cudaStream_t s) {
    const int np = (int)L.parts.size();
    if (np == 0) return;
    // the split costs a second launch: worth it for the FP64 sums, and in FP32 for large meshes
    // (measured: 642-vertex capsule FP32 slower split, 2562-vertex RBC and every FP64 case faster)
    const bool big = L.storage == BIB_STORAGE_F64 || L.max_nt >= 4096;
    const int split = big ? std::min(kMaxUpdateSplit, membrane_split(np, L.max_nt, 256)) : 1;
    if (split > 1 && L.upd_partial) {
        const IbView v = single_view(L, -1);
        const size_t sm = L.storage == BIB_STORAGE_F64 ? 0 : 3 * sizeof(float) * L.max_nv;
        if (L.storage == BIB_STORAGE_F64) {
            k_update_partial<double><<<dim3(np, split), 256, sm, s>>>(L.pdev, v, L.upd_partial);
            k_update_finish<double><<<np, 256, 0, s>>>(L.pdev, v, L.upd_partial, split);
        } else {
            k_update_partial<float><<<dim3(np, split), 256, sm, s>>>(L.pdev, v, L.upd_partial);
            k_update_finish<float><<<np, 256, 0, s>>>(L.pdev, v, L.upd_partial, split);
        }
        return;
    }
    update_any<false>(L.storage, L.pdev, np, single_view(L, -1), nullptr, L.max_nv, s);
}

void launch_membrane_batch(const BatchLaunch& B, int block, cudaStream_t s) {
    if (B.nparts == 0) return;
    membrane_any<true>(B.storage, B.parts, B.nparts, IbView{}, B.views, B.membrane_smem, block, s);
}
void launch_spread_batch(const BatchLaunch& B, cudaStream_t s) {
    if (B.nvert == 0) return;
    spread_any<true>(B.storage, B.dirac, IbView{}, B.views, B.vinst, B.nvert, s);
}
void launch_interpolate_batch(const BatchLaunch& B, cudaStream_t s) {
    if (B.nvert == 0) return;
    interpolate_any<true>(B.storage, B.dirac, IbView{}, B.views, B.vinst, B.nvert, s);
}
void launch_update_batch(const BatchLaunch& B, cudaStream_t s) {
    if (B.nparts == 0) return;
    update_any<true>(B.storage, B.parts, B.nparts, IbView{}, B.views, B.max_nv, s);
}

void launch_spread(const Lattice& L, int fbuf, cudaStream_t s, bool record) {
    if (L.nvert == 0) return;
    const unsigned g = (L.nvert + 127) / 128;
    const double* pos = L.pos[L.pcur];
    int4* lo = record ? L.spread_lo[fbuf] : nullptr;
    if (L.ib.spread_mode == BIB_SPREAD_DETERMINISTIC) {
        const int sup = L.ib.dirac == BIB_DIRAC_PESKIN ? 4 : 3;
        const int64_t ne = (int64_t)L.nvert * sup * sup * sup;
        k_spread_keys<<<g, 128, 0, s>>>(L.d, L.ib, L.nvert, pos, L.sort_keys[0], L.sort_ids[0], lo);
        size_t tb = L.sort_temp_bytes;
        cub::DeviceRadixSort::SortPairs(L.sort_temp, tb, L.sort_keys[0], L.sort_keys[1], L.sort_ids[0], L.sort_ids[1],
                                        (int)ne, 0, key_bits(L.d.n), s);
        const unsigned ge = (unsigned)((ne + 127) / 128);
        if (L.storage == BIB_STORAGE_F64)
            k_spread_reduce<double><<<ge, 128, 0, s>>>(L.d, L.ib, ne, L.sort_keys[1], L.sort_ids[1], pos, L.force, (double*)L.F[fbuf]);
        else
            k_spread_reduce<float><<<ge, 128, 0, s>>>(L.d, L.ib, ne, L.sort_keys[1], L.sort_ids[1], pos, L.force, (float*)L.F[fbuf]);
        return;
    }
    IbView v = single_view(L, fbuf);
    v.spread_lo = lo;
    spread_any<false>(L.storage, L.ib.dirac, v, nullptr, nullptr, L.nvert, s);
}

// Phase field of the membranes at pos (the positions of the current step's end): z-rays of
// every triangle, then the per-column parity fill.  count must be zero on entry (it is left
// zero); a column with more than cap crossings, or a triangle wider than the lattice, sets
// *overflow (the column keeps its first cap crossings, the triangle casts no rays).
void launch_voxelize(const Lattice& L, const double* pos, cudaStream_t s) {
    if (!L.phase || L.parts.empty()) return;
    k_voxel_rays<<<(int)L.parts.size(), 128, 0, s>>>(L.d, L.pdev, pos, L.vox_count, L.vox_z, kVoxelCap, L.vox_err);
    const int64_t ncol = (int64_t)L.d.nx * L.d.ny;
    k_voxel_fill<<<(unsigned)((ncol + 127) / 128), 128, 0, s>>>(L.d, L.vox_count, L.vox_z, kVoxelCap, L.phase);
}

// ---- RBC shape calibration: RBCParticle::relax_nodes (RBCParticle.hh:318-342) ----
// One iteration of shrink_rbc_volume (progs/common/calibrate_rbc_shape.h:25-33) for the single
// particle of L: vol_desired of iteration it (while it <= n_it) into the particle's parameters,
// node masses M_i = sum over the triangles at i (in triangle order) of area/3, vel += force/M -
// damping vel, pos_next = pos + vel.  The forces of pos_next are computed by the membrane
// kernel afterwards, with the new vol_desired.  Operations are rounded one by one (no
// contraction) in the reference's order.  One block; *iter counts the iterations.
__global__ void __launch_bounds__(256) k_rbc_relax(ParticleDev* P, const double* __restrict__ pos,
                                                   double* __restrict__ pos_next, double* __restrict__ vel,
                                                   const double* __restrict__ force, int nv, double damping,
                                                   long long* iter, long long n_it, double vol_start, double vol_final) {
    const long long it = *iter;
    const ParticleDev& p = *P;
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        double M = 0.0;
        for (int e = p.inc_off[i]; e < p.inc_off[i + 1]; ++e) {
            const int code = p.inc[e];
            if ((code >> 29) != 1) continue;  // triangles only
            const int t = code & ((1 << 29) - 1);
            const int i0 = p.tri[3 * t], i1 = p.tri[3 * t + 1], i2 = p.tri[3 * t + 2];
            const double ax = pos[3 * i0], ay = pos[3 * i0 + 1], az = pos[3 * i0 + 2];
            const double ux = __dsub_rn(pos[3 * i1], ax), uy = __dsub_rn(pos[3 * i1 + 1], ay),
                         uz = __dsub_rn(pos[3 * i1 + 2], az);
            const double wx = __dsub_rn(pos[3 * i2], ax), wy = __dsub_rn(pos[3 * i2 + 1], ay),
                         wz = __dsub_rn(pos[3 * i2 + 2], az);
            const double cx = __dsub_rn(__dmul_rn(uy, wz), __dmul_rn(uz, wy));
            const double cy = __dsub_rn(__dmul_rn(uz, wx), __dmul_rn(ux, wz));
            const double cz = __dsub_rn(__dmul_rn(ux, wy), __dmul_rn(uy, wx));
            const double n2 = __dadd_rn(__dadd_rn(__dmul_rn(cx, cx), __dmul_rn(cy, cy)), __dmul_rn(cz, cz));
            M = __dadd_rn(M, __ddiv_rn(__dmul_rn(0.5, __dsqrt_rn(n2)), 3.0));
        }
        for (int k = 0; k < 3; ++k) {
            const double v = vel[3 * i + k];
            const double nvk = __dadd_rn(v, __dsub_rn(__ddiv_rn(force[3 * i + k], M), __dmul_rn(damping, v)));
            vel[3 * i + k] = nvk;
            pos_next[3 * i + k] = __dadd_rn(pos[3 * i + k], nvk);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (it <= n_it)
            P->prm[BIB_P_VOL_DESIRED] =
                __dadd_rn(vol_start, __dmul_rn(__ddiv_rn((double)it, (double)n_it), __dsub_rn(vol_final, vol_start)));
        *iter = it + 1;
    }
}

void launch_rbc_relax(const Lattice& L, double damping, long long* iter, long long n_it, double vol_start,
                      double vol_final, cudaStream_t s) {
    k_rbc_relax<<<1, 256, 0, s>>>(L.pdev, L.pos[L.pcur], L.pos[1 - L.pcur], L.vel, L.force, L.nvert, damping, iter,
                                   n_it, vol_start, vol_final);
}

}  // namespace bib
