// Lattice addressing shared by the collide-and-stream kernels: finite-difference wall
// buffer, source cells of the pull gather and the moving-wall bounce-back term.
#pragma once

#include "d3q19.cuh"

namespace bib {

__device__ __forceinline__ bool fd_wall_node(const LatticeDesc& d, int y) { return d.fd_walls && (y == 0 || y == d.ny - 1); }

__device__ __forceinline__ int64_t wall_index(const LatticeDesc& d, int side, int x, int z) {
    return ((int64_t)side * d.nz + z) * d.nx + x;
}
__device__ __forceinline__ int64_t wall_stride(const LatticeDesc& d) { return 2LL * d.nz * d.nx; }

// Source cell of population i arriving at (x, y, z).  Returns the cell index, or -1 if
// the source lies behind a wall; `face` then tells which wall (0 y-, 1 y+, 2 z-, 3 z+).
__device__ __forceinline__ int64_t source_cell(const LatticeDesc& d, int i, int x, int y, int z, int& face) {
    int xs = x - cx(i), ys = y - cy(i), zs = z - cz(i);
    face = -1;
    xs = (int)wrap_index(xs, d.nx);
    if (d.py) ys = (int)wrap_index(ys, d.ny);
    else if (ys < 0 || ys >= d.ny) face = ys < 0 ? 0 : 1;
    if (d.pz) zs = (int)wrap_index(zs, d.nz);
    else if (face < 0 && (zs < 0 || zs >= d.nz)) face = zs < 0 ? 2 : 3;
    if (face >= 0) return -1;
    return xs + (int64_t)d.nx * (ys + (int64_t)d.ny * zs);
}

template <class C>
__device__ __forceinline__ C moving_wall_term(const LatticeDesc& d, int i, int face) {
    const C cu = C(cx(i)) * (C)d.wall_u[face][0] + C(cy(i)) * (C)d.wall_u[face][1] + C(cz(i)) * (C)d.wall_u[face][2];
    return C(6) * weight<C>(i) * cu;
}


// The velocity field is stored as four values per cell (ux, uy, uz, 0): one aligned vector
// access per cell for the interpolation's 27 / 64-node gathers (FP64, FP32, or FP16 for FP16
// population storage).
template <class FT>
__device__ __forceinline__ void store_u(FT* u, int64_t k, FT a, FT b, FT c);
template <>
__device__ __forceinline__ void store_u<float>(float* u, int64_t k, float a, float b, float c) {
    reinterpret_cast<float4*>(u)[k] = make_float4(a, b, c, 0.0f);
}
template <>
__device__ __forceinline__ void store_u<double>(double* u, int64_t k, double a, double b, double c) {
    double2* q = reinterpret_cast<double2*>(u) + 2 * k;
    q[0] = make_double2(a, b);
    q[1] = make_double2(c, 0.0);
}
// FP16 storage: four halves (8 bytes) per cell
template <>
__device__ __forceinline__ void store_u<__half>(__half* u, int64_t k, __half a, __half b, __half c) {
    const __half2 ab = __halves2half2(a, b), c0 = __halves2half2(c, __ushort_as_half(0));
    reinterpret_cast<uint2*>(u)[k] = make_uint2(*reinterpret_cast<const unsigned*>(&ab), *reinterpret_cast<const unsigned*>(&c0));
}

// The velocity from the compute type: FP16 converts two components per instruction.
template <class UT, class C>
__device__ __forceinline__ void store_u_from(UT* u, int64_t k, C a, C b, C c) {
    store_u<UT>(u, k, (UT)a, (UT)b, (UT)c);
}
template <>
__device__ __forceinline__ void store_u_from<__half, float>(__half* u, int64_t k, float a, float b, float c) {
    const __half2 ab = __floats2half2_rn(a, b), c0 = __floats2half2_rn(c, 0.0f);
    reinterpret_cast<uint2*>(u)[k] = make_uint2(*reinterpret_cast<const unsigned*>(&ab), *reinterpret_cast<const unsigned*>(&c0));
}

// BounceBack::collide (core/dynamics.hh:763-770): each population swaps with its opposite.
template <class C>
__device__ __forceinline__ void bounce_back_cell(C* f) {
#pragma unroll
    for (int i = 1; i <= 9; ++i) {
        const C t = f[i];
        f[i] = f[i + 9];
        f[i + 9] = t;
    }
}

// Row (y, z) lies next to a wall or is a finite-difference wall row: its gather needs the
// per-population face tests; every other row streams from its 18 neighbours unchanged.
__device__ __forceinline__ bool row_special(const LatticeDesc& d, int y, int z) {
    return fd_wall_node(d, y) || (!d.py && (y == 0 || y == d.ny - 1)) || (!d.pz && (z == 0 || z == d.nz - 1));
}

// Wall face behind the source of population i arriving in row (y, z), or -1 if the source
// row (y - c_iy, z - c_iz) is inside the domain (after periodic wrap, returned in srow).
__device__ __forceinline__ int source_row(const LatticeDesc& d, int i, int y, int z, int64_t& srow) {
    int ys = y - cy(i), zs = z - cz(i), face = -1;
    if (d.py) ys = (int)wrap_index(ys, d.ny);
    else if (ys < 0 || ys >= d.ny) face = ys < 0 ? 0 : 1;
    if (d.pz) zs = (int)wrap_index(zs, d.nz);
    else if (face < 0 && (zs < 0 || zs >= d.nz)) face = zs < 0 ? 2 : 3;
    srow = face >= 0 ? -1 : (int64_t)ys + (int64_t)d.ny * zs;
    return face;
}

// Two neighbouring cells of one population row (x even), as one vector access.
template <class T>
struct Pair;
template <>
struct Pair<__half> {
    static __device__ __forceinline__ void load(const __half* p, float inv, float& a, float& b) {
        const float2 v = __half22float2(__ldg(reinterpret_cast<const __half2*>(p)));
        a = v.x * inv;
        b = v.y * inv;
    }
    static __device__ __forceinline__ void store(__half* p, float a, float b, float s) {
        *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a * s, b * s);
    }
    // scaled values as stored (f-bar * S)
    static __device__ __forceinline__ void load_raw(const __half* p, float& a, float& b) {
        const float2 v = __half22float2(__ldg(reinterpret_cast<const __half2*>(p)));
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void store_raw(__half* p, float a, float b) {
        *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b);
    }
    static __device__ __forceinline__ float load1_raw(const __half* p) { return __half2float(__ldg(p)); }
};
template <>
struct Pair<float> {
    static __device__ __forceinline__ void load(const float* p, float, float& a, float& b) {
        const float2 v = __ldg(reinterpret_cast<const float2*>(p));
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void store(float* p, float a, float b, float) {
        *reinterpret_cast<float2*>(p) = make_float2(a, b);
    }
    static __device__ __forceinline__ void load_raw(const float* p, float& a, float& b) { load(p, 1.0f, a, b); }
    static __device__ __forceinline__ void store_raw(float* p, float a, float b) { store(p, a, b, 1.0f); }
    static __device__ __forceinline__ float load1_raw(const float* p) { return __ldg(p); }
};
template <>
struct Pair<double> {
    static __device__ __forceinline__ void load(const double* p, float, double& a, double& b) {
        const double2 v = __ldg(reinterpret_cast<const double2*>(p));
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void store(double* p, double a, double b, float) {
        *reinterpret_cast<double2*>(p) = make_double2(a, b);
    }
};

template <class FT>
__device__ __forceinline__ void load2(const FT* p, FT& a, FT& b);
template <>
__device__ __forceinline__ void load2<float>(const float* p, float& a, float& b) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    a = v.x;
    b = v.y;
}
template <>
__device__ __forceinline__ void load2<double>(const double* p, double& a, double& b) {
    const double2 v = __ldg(reinterpret_cast<const double2*>(p));
    a = v.x;
    b = v.y;
}
template <class FT>
__device__ __forceinline__ void store2(FT* p, FT a, FT b);
template <>
__device__ __forceinline__ void store2<float>(float* p, float a, float b) {
    *reinterpret_cast<float2*>(p) = make_float2(a, b);
}
template <>
__device__ __forceinline__ void store2<double>(double* p, double a, double b) {
    *reinterpret_cast<double2*>(p) = make_double2(a, b);
}

}  // namespace bib
