// Lattice kernels: fused collide-and-stream, finite-difference velocity walls,
// velocity field, equilibrium initialisation and host-format conversion.
//
// Data layout in HBM: one array per population (structure of arrays), x fastest,
// cell k = x + nx*(y + ny*z), population i at f[i*stride + k].  The stored state is
// post-streaming (Palabos semantics), so streaming is a push: a cell reads its own 19
// populations (coalesced), collides in registers and writes each population into the
// neighbour it moves to (x-shifted writes stay coalesced at sector level).
#include <cstdio>

#include "d3q19.cuh"

namespace bib {

namespace {

template <class T>
__global__ void __launch_bounds__(256) k_collide_stream(LatticeDesc d, const T* __restrict__ fin, T* __restrict__ fout,
                                                         const typename Store<T>::F* __restrict__ F,
                                                         const uint8_t* __restrict__ phase, int coll) {
    using C = typename Store<T>::C;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= d.nx) return;
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    C f[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = Store<T>::load(fin + i * d.stride + k, d.inv_scale);
    C Fc[3];
    Fc[0] = (C)__ldg(F + k);
    Fc[1] = (C)__ldg(F + d.stride + k);
    Fc[2] = (C)__ldg(F + 2 * d.stride + k);
    C omega = (C)d.omega_c0;
    if (d.use_phase && phase[k]) omega = (C)d.omega_c1;
    if (coll == BIB_COLLISION_BGK_GUO_VOF) {
        collide<C, BIB_COLLISION_BGK_GUO_VOF>(f, Fc, omega, C(0));
    } else if (coll == BIB_COLLISION_BGK) {
        collide<C, BIB_COLLISION_BGK>(f, Fc, (C)d.omega, C(0));
    } else {
        const C om = (C)d.omega;
        const C omm = C(1) / ((C)d.trt_magic / (C(1) / om - C(0.5)) + C(0.5));
        collide<C, BIB_COLLISION_TRT>(f, Fc, om, omm);
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        int xd = x + cx(i), yd = y + cy(i), zd = z + cz(i);
        int face = -1;
        if (d.px) xd = (int)wrap_index(xd, d.nx);
        else if (xd < 0 || xd >= d.nx) face = 4;
        if (d.py) yd = (int)wrap_index(yd, d.ny);
        else if (yd < 0 || yd >= d.ny) face = yd < 0 ? 0 : 1;
        if (d.pz) zd = (int)wrap_index(zd, d.nz);
        else if (face < 0 && (zd < 0 || zd >= d.nz)) face = zd < 0 ? 2 : 3;
        if (face < 0) {
            const int64_t kd = xd + (int64_t)d.nx * (yd + (int64_t)d.ny * zd);
            Store<T>::store(fout + i * d.stride + kd, f[i], d.scale);
        } else {
            // The population leaves the domain.  Halfway bounce-back returns it reversed
            // to its own node with the moving-wall term -6 t_i (c_i . u_w) (rho_w = 1).
            // FD velocity walls drop it: the wall processor rebuilds the wall node.
            const int wall = face <= 1 ? d.wall_y : (face <= 3 ? d.wall_z : BIB_WALL_NONE);
            if (wall == BIB_WALL_HALFWAY_BB) {
                const C cu = C(cx(i)) * (C)d.wall_u[face][0] + C(cy(i)) * (C)d.wall_u[face][1] + C(cz(i)) * (C)d.wall_u[face][2];
                Store<T>::store(fout + opposite(i) * d.stride + k, f[i] - C(6) * weight<C>(i) * cu, d.scale);
            }
        }
    }
}

// PlaneFdBoundaryFunctional3D::processCell on the y walls,
// src/boundaryCondition/finiteDifferenceBoundaryProcessor3D.hh:68-115: density from the
// known populations (VelocityDirichletBoundaryDynamics::computeRhoBar,
// boundaryDynamics.hh:631-663), one-sided normal velocity derivative
// (finiteDifference3D.h:67-82; tangential derivatives vanish for a uniform wall
// velocity), regularised reconstruction of all 19 populations.
template <class T>
__global__ void k_fd_walls(LatticeDesc d, T* __restrict__ f, const typename Store<T>::F* __restrict__ F) {
    using C = typename Store<T>::C;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    const int side = blockIdx.z;
    if (x >= d.nx) return;
    const int y = side == 0 ? 0 : d.ny - 1;
    const int orientation = side == 0 ? -1 : 1;
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    const int64_t k1 = x + (int64_t)d.nx * (y - orientation + (int64_t)d.ny * z);
    C fc[Q], f1[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        fc[i] = Store<T>::load(f + i * d.stride + k, d.inv_scale);
        f1[i] = Store<T>::load(f + i * d.stride + k1, d.inv_scale);
    }
    const C Fy = (C)F[d.stride + k];
    C F1[3] = {(C)F[k1], (C)F[d.stride + k1], (C)F[2 * d.stride + k1]};
    const C uw[3] = {(C)d.wall_u[side][0], (C)d.wall_u[side][1], (C)d.wall_u[side][2]};
    C rhoOnWall = 0, rhoNormal = 0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        if (cy(i) == 0) rhoOnWall += fc[i];
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        if (cy(i) == orientation) rhoNormal += fc[i];
    }
    const C velNormal = C(orientation) * (uw[1] - C(0.5) * Fy);
    const C rhoBarW = (C(2) * rhoNormal + rhoOnWall - velNormal) / (C(1) + velNormal);
    const C rho = rhoBarW + C(1);
    C u1[3];
    velocity_with_force(f1, F1, u1);
    C dy_u[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) dy_u[a] = C(-orientation) * (u1[a] - uw[a]);
    const C sToPi = -rho / C(3) / (C)d.omega;
    // pi: xx, xy, xz, yy, yz, zz with the tangential derivatives equal to zero
    const C pi[6] = {C(0), dy_u[0] * sToPi, C(0), C(2) * dy_u[1] * sToPi, dy_u[2] * sToPi, C(0)};
    C j[3] = {rho * uw[0], rho * uw[1], rho * uw[2]};
    const C jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    const C rhoBar = rho - C(1);
    const C invRho = C(1) / (rhoBar + C(1));
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        // fromPiToFneq, src/latticeBoltzmann/offEquilibriumTemplates.h:91-115
        const C c0 = C(cx(i)), c1 = C(cy(i)), c2 = C(cz(i));
        const C cs2 = C(1) / C(3);
        C fneq = C(0);
        fneq += pi[0] * (c0 * c0 - cs2);
        fneq += pi[1] * C(2) * c0 * c1;
        fneq += pi[2] * C(2) * c0 * c2;
        fneq += pi[3] * (c1 * c1 - cs2);
        fneq += pi[4] * C(2) * c1 * c2;
        fneq += pi[5] * (c2 * c2 - cs2);
        fneq *= weight<C>(i) * C(3) * C(3) / C(2);
        Store<T>::store(f + i * d.stride + k, bgk_equilibrium<C>(i, rhoBar, invRho, j, jSqr) + fneq, d.scale);
    }
}

__device__ __forceinline__ bool is_fd_wall(const LatticeDesc& d, int y, int z) {
    (void)z;
    return !d.py && d.wall_y == BIB_WALL_FD_VELOCITY && (y == 0 || y == d.ny - 1);
}

template <class T>
__global__ void k_velocity(LatticeDesc d, const T* __restrict__ f, const typename Store<T>::F* __restrict__ F,
                           double* __restrict__ u) {
    using C = typename Store<T>::C;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= d.nx) return;
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    if (is_fd_wall(d, y, z)) {
        const int side = y == 0 ? 0 : 1;
        for (int a = 0; a < 3; ++a) u[a * d.n + k] = d.wall_u[side][a];
        return;
    }
    C fc[Q], Fc[3], uc[3];
#pragma unroll
    for (int i = 0; i < Q; ++i) fc[i] = Store<T>::load(f + i * d.stride + k, d.inv_scale);
    for (int a = 0; a < 3; ++a) Fc[a] = (C)F[a * d.stride + k];
    velocity_with_force(fc, Fc, uc);
    for (int a = 0; a < 3; ++a) u[a * d.n + k] = (double)uc[a];
}

// iniCellAtEquilibrium, src/core/cell.hh:124-132
template <class T>
__global__ void k_init_eq(LatticeDesc d, T* __restrict__ f, const double* __restrict__ rho, const double* __restrict__ u) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    const double r = rho ? rho[k] : 1.0;
    double j[3] = {u[k] * r, u[d.n + k] * r, u[2 * d.n + k] * r};
    const double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    const double rhoBar = r - 1.0;
    const double invRho = 1.0 / (rhoBar + 1.0);
#pragma unroll
    for (int i = 0; i < Q; ++i)
        Store<T>::store(f + i * d.stride + k, (typename Store<T>::C)bgk_equilibrium<double>(i, rhoBar, invRho, j, jSqr), d.scale);
}

template <class T>
__global__ void k_import(LatticeDesc d, T* __restrict__ f, const double* __restrict__ src) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    for (int i = 0; i < Q; ++i) Store<T>::store(f + i * d.stride + k, (typename Store<T>::C)src[i * d.n + k], d.scale);
}

template <class T>
__global__ void k_export(LatticeDesc d, const T* __restrict__ f, double* __restrict__ dst) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    for (int i = 0; i < Q; ++i) dst[i * d.n + k] = (double)Store<T>::load(f + i * d.stride + k, d.inv_scale);
}

template <class FT>
__global__ void k_force_import(LatticeDesc d, FT* __restrict__ F, const double* __restrict__ src) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    for (int a = 0; a < 3; ++a) F[a * d.stride + k] = (FT)src[a * d.n + k];
}

template <class FT>
__global__ void k_force_export(LatticeDesc d, const FT* __restrict__ F, double* __restrict__ dst) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    for (int a = 0; a < 3; ++a) dst[a * d.n + k] = (double)F[a * d.stride + k];
}

template <class FT>
__global__ void k_force_fill(LatticeDesc d, FT* __restrict__ F) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= d.stride) return;
    F[k] = (FT)d.body[0];
    F[d.stride + k] = (FT)d.body[1];
    F[2 * d.stride + k] = (FT)d.body[2];
}

__global__ void k_phase_import(LatticeDesc d, uint8_t* __restrict__ ph, const double* __restrict__ src) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    ph[k] = src[k] >= 0.5 ? 1 : 0;
}

template <class T>
__global__ void k_nan_scan(LatticeDesc d, const T* __restrict__ f, int* flag) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    bool bad = false;
    for (int i = 0; i < Q; ++i) {
        const float v = (float)Store<T>::load(f + i * d.stride + k, d.inv_scale);
        bad |= !isfinite(v);
    }
    if (bad) atomicOr(flag, 1);
}

inline dim3 row_grid(const LatticeDesc& d, int bx) { return dim3((d.nx + bx - 1) / bx, d.ny, d.nz); }
inline int row_block(const LatticeDesc& d) { return d.nx >= 256 ? 256 : (d.nx >= 128 ? 128 : (d.nx >= 64 ? 64 : 32)); }
inline unsigned lin_grid(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

template <class T>
void collide_stream_t(const Lattice& L, cudaStream_t s) {
    const int bx = row_block(L.d);
    using FT = typename Store<T>::F;
    k_collide_stream<T><<<row_grid(L.d, bx), bx, 0, s>>>(L.d, (const T*)L.f[L.cur], (T*)L.f[1 - L.cur], (const FT*)L.F,
                                                           L.phase, L.d.collision);
}

}  // namespace

void launch_collide_stream(const Lattice& L, cudaStream_t s) {
    if (L.storage == BIB_STORAGE_F64) collide_stream_t<double>(L, s);
    else if (L.storage == BIB_STORAGE_F32) collide_stream_t<float>(L, s);
    else collide_stream_t<__half>(L, s);
}

void launch_fd_walls(const Lattice& L, void* f, cudaStream_t s) {
    if (L.d.py || L.d.wall_y != BIB_WALL_FD_VELOCITY) return;
    const int bx = row_block(L.d);
    dim3 g((L.d.nx + bx - 1) / bx, L.d.nz, 2);
    if (L.storage == BIB_STORAGE_F64) k_fd_walls<double><<<g, bx, 0, s>>>(L.d, (double*)f, (const double*)L.F);
    else if (L.storage == BIB_STORAGE_F32) k_fd_walls<float><<<g, bx, 0, s>>>(L.d, (float*)f, (const float*)L.F);
    else k_fd_walls<__half><<<g, bx, 0, s>>>(L.d, (__half*)f, (const float*)L.F);
}

void launch_velocity(const Lattice& L, double* u, cudaStream_t s) {
    const int bx = row_block(L.d);
    const void* f = L.f[L.cur];
    if (L.storage == BIB_STORAGE_F64) k_velocity<double><<<row_grid(L.d, bx), bx, 0, s>>>(L.d, (const double*)f, (const double*)L.F, u);
    else if (L.storage == BIB_STORAGE_F32) k_velocity<float><<<row_grid(L.d, bx), bx, 0, s>>>(L.d, (const float*)f, (const float*)L.F, u);
    else k_velocity<__half><<<row_grid(L.d, bx), bx, 0, s>>>(L.d, (const __half*)f, (const float*)L.F, u);
}

void launch_init_equilibrium(const Lattice& L, void* f, const double* rho, const double* u, cudaStream_t s) {
    const unsigned g = lin_grid(L.d.n, 256);
    if (L.storage == BIB_STORAGE_F64) k_init_eq<double><<<g, 256, 0, s>>>(L.d, (double*)f, rho, u);
    else if (L.storage == BIB_STORAGE_F32) k_init_eq<float><<<g, 256, 0, s>>>(L.d, (float*)f, rho, u);
    else k_init_eq<__half><<<g, 256, 0, s>>>(L.d, (__half*)f, rho, u);
}

void launch_import_soa(const Lattice& L, void* f, const double* src, cudaStream_t s) {
    const unsigned g = lin_grid(L.d.n, 256);
    if (L.storage == BIB_STORAGE_F64) k_import<double><<<g, 256, 0, s>>>(L.d, (double*)f, src);
    else if (L.storage == BIB_STORAGE_F32) k_import<float><<<g, 256, 0, s>>>(L.d, (float*)f, src);
    else k_import<__half><<<g, 256, 0, s>>>(L.d, (__half*)f, src);
}

void launch_export_soa(const Lattice& L, const void* f, double* dst, cudaStream_t s) {
    const unsigned g = lin_grid(L.d.n, 256);
    if (L.storage == BIB_STORAGE_F64) k_export<double><<<g, 256, 0, s>>>(L.d, (const double*)f, dst);
    else if (L.storage == BIB_STORAGE_F32) k_export<float><<<g, 256, 0, s>>>(L.d, (const float*)f, dst);
    else k_export<__half><<<g, 256, 0, s>>>(L.d, (const __half*)f, dst);
}

void launch_force_import(const Lattice& L, const double* src, cudaStream_t s) {
    const unsigned g = lin_grid(L.d.n, 256);
    if (L.storage == BIB_STORAGE_F64) k_force_import<double><<<g, 256, 0, s>>>(L.d, (double*)L.F, src);
    else k_force_import<float><<<g, 256, 0, s>>>(L.d, (float*)L.F, src);
}

void launch_force_export(const Lattice& L, double* dst, cudaStream_t s) {
    const unsigned g = lin_grid(L.d.n, 256);
    if (L.storage == BIB_STORAGE_F64) k_force_export<double><<<g, 256, 0, s>>>(L.d, (const double*)L.F, dst);
    else k_force_export<float><<<g, 256, 0, s>>>(L.d, (const float*)L.F, dst);
}

void launch_force_fill(const Lattice& L, cudaStream_t s) {
    const size_t fsz = L.storage == BIB_STORAGE_F64 ? sizeof(double) : sizeof(float);
    if (L.d.body[0] == 0.0 && L.d.body[1] == 0.0 && L.d.body[2] == 0.0) {
        cudaMemsetAsync(L.F, 0, 3 * L.d.stride * fsz, s);
        return;
    }
    const unsigned g = lin_grid(L.d.stride, 256);
    if (L.storage == BIB_STORAGE_F64) k_force_fill<double><<<g, 256, 0, s>>>(L.d, (double*)L.F);
    else k_force_fill<float><<<g, 256, 0, s>>>(L.d, (float*)L.F);
}

void launch_phase_import(const Lattice& L, const double* src, cudaStream_t s) {
    k_phase_import<<<lin_grid(L.d.n, 256), 256, 0, s>>>(L.d, L.phase, src);
}

void launch_nan_scan(const Lattice& L, int* flag, cudaStream_t s) {
    const unsigned g = lin_grid(L.d.n, 256);
    const void* f = L.f[L.cur];
    if (L.storage == BIB_STORAGE_F64) k_nan_scan<double><<<g, 256, 0, s>>>(L.d, (const double*)f, flag);
    else if (L.storage == BIB_STORAGE_F32) k_nan_scan<float><<<g, 256, 0, s>>>(L.d, (const float*)f, flag);
    else k_nan_scan<__half><<<g, 256, 0, s>>>(L.d, (const __half*)f, flag);
}

}  // namespace bib
