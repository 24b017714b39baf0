// Lattice kernels: fused pull collide-and-stream (+ velocity field), finite-difference
// velocity walls, state import / export and equilibrium initialisation.
//
// Data layout in HBM: one array per population (structure of arrays), x fastest,
// cell k = x + nx*(y + ny*z), population i at f[i*stride + k].  The buffers hold
// post-collision populations f*(x); the post-streaming state (the reference's state
// between steps) is gathered: f_i(x) = f*_i(x - c_i), periodic by index wrap, halfway
// bounce-back f_i(x) = f*_opp(i)(x) + 6 t_i (c_i . u_wall) where x - c_i lies behind a
// wall, and the nodes of finite-difference velocity walls read a separate wall buffer.
#include <algorithm>

#include "lattice_common.cuh"

namespace bib {

namespace {

// Post-streaming populations of one cell.
template <class T>
__device__ __forceinline__ void gather(const LatticeDesc& d, const T* __restrict__ f, const T* __restrict__ wall, int x,
                                       int y, int z, int64_t k, typename Store<T>::C* out) {
    using C = typename Store<T>::C;
    if (fd_wall_node(d, y)) {
        const int64_t wk = wall_index(d, y == 0 ? 0 : 1, x, z), ws = wall_stride(d);
#pragma unroll
        for (int i = 0; i < Q; ++i) out[i] = Store<T>::load(wall + i * ws + wk, d.inv_scale);
        return;
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        int face;
        const int64_t s = source_cell(d, i, x, y, z, face);
        if (s >= 0) out[i] = Store<T>::load(f + i * d.stride + s, d.inv_scale);
        else out[i] = Store<T>::load(f + opposite(i) * d.stride + k, d.inv_scale) + moving_wall_term<C>(d, i, face);
    }
}

// Inverse of gather for a single population: where the value f_i(x) of a post-streaming
// state has to be stored so that the next gather returns it.
template <class T>
__device__ __forceinline__ void scatter_canonical(const LatticeDesc& d, T* __restrict__ f, T* __restrict__ wall, int i, int x,
                                                  int y, int z, int64_t k, typename Store<T>::C v) {
    using C = typename Store<T>::C;
    if (fd_wall_node(d, y)) {
        Store<T>::store(wall + i * wall_stride(d) + wall_index(d, y == 0 ? 0 : 1, x, z), v, d.scale);
        return;
    }
    int face;
    const int64_t s = source_cell(d, i, x, y, z, face);
    if (s >= 0) Store<T>::store(f + i * d.stride + s, v, d.scale);
    else Store<T>::store(f + opposite(i) * d.stride + k, v - moving_wall_term<C>(d, i, face), d.scale);
}

template <class T, bool COUPLED>
__global__ void __launch_bounds__(256) k_collide_stream(LatticeDesc d, const T* __restrict__ fin, T* __restrict__ fout,
                                                         const T* __restrict__ wall,
                                                         const typename Store<T>::F* __restrict__ Fcol,
                                                         typename Store<T>::F* __restrict__ Fprev,
                                                         typename Store<T>::U* __restrict__ u_out,
                                                         const uint8_t* __restrict__ phase,
                                                         const uint8_t* __restrict__ celltype, int coll) {
    using C = typename Store<T>::C;
    using FT = typename Store<T>::F;
    using UT = typename Store<T>::U;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= d.nx) return;
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    C f[Q];
    gather<T>(d, fin, wall, x, y, z, k, f);
    const int ctype = d.has_types ? celltype[k] : BIB_CELL_FLUID;
    if (ctype != BIB_CELL_FLUID) {  // BounceBack / NoDynamics node: no collision, zero velocity
        if (COUPLED) {
            store_u<UT>(u_out, k, (UT)0.0f, (UT)0.0f, (UT)0.0f);
            if (Fprev)
                for (int c = 0; c < 3; ++c) Fprev[c * d.stride + k] = (FT)d.body[c];
        }
        if (ctype == BIB_CELL_BOUNCE_BACK) bounce_back_cell(f);
#pragma unroll
        for (int i = 0; i < Q; ++i) Store<T>::store(fout + i * d.stride + k, f[i], d.scale);
        return;
    }
    if (COUPLED) {
        // computeVelocity of the current state (externalForceDynamics.hh:59-74; the wall
        // nodes give their imposed velocity, boundaryDynamics.hh:316-322), with the force of
        // the previous collision; that force buffer is then reset to the body force so the
        // next step can spread into it (setExternalVector).  Without Fprev (sparse force
        // reset) the velocity takes the body force and the interpolation adds the rest.
        C u[3];
        if (fd_wall_node(d, y)) {
            const int side = y == 0 ? 0 : 1;
            u[0] = (C)d.wall_u[side][0];
            u[1] = (C)d.wall_u[side][1];
            u[2] = (C)d.wall_u[side][2];
        } else {
            C Fp[3] = {(C)d.body[0], (C)d.body[1], (C)d.body[2]};
            if (Fprev) {
                Fp[0] = (C)Fprev[k];
                Fp[1] = (C)Fprev[d.stride + k];
                Fp[2] = (C)Fprev[2 * d.stride + k];
            }
            velocity_with_force(f, Fp, u);
        }
        store_u<UT>(u_out, k, (UT)u[0], (UT)u[1], (UT)u[2]);
        if (Fprev) {
            Fprev[k] = (FT)d.body[0];
            Fprev[d.stride + k] = (FT)d.body[1];
            Fprev[2 * d.stride + k] = (FT)d.body[2];
        }
    }
    C Fc[3] = {(C)__ldg(Fcol + k), (C)__ldg(Fcol + d.stride + k), (C)__ldg(Fcol + 2 * d.stride + k)};
    if (coll == BIB_COLLISION_BGK_GUO_VOF) {
        C omega = (C)d.omega_c0;
        if (d.use_phase && phase[k]) omega = (C)d.omega_c1;
        collide_unscaled<C, BIB_COLLISION_BGK_GUO_VOF>(f, Fc, omega, C(0));
    } else if (coll == BIB_COLLISION_BGK) {
        collide_unscaled<C, BIB_COLLISION_BGK>(f, Fc, (C)d.omega, C(0));
    } else {
        const C om = (C)d.omega;
        const C omm = C(1) / ((C)d.trt_magic / (C(1) / om - C(0.5)) + C(0.5));
        collide_unscaled<C, BIB_COLLISION_TRT>(f, Fc, om, omm);
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) Store<T>::store(fout + i * d.stride + k, f[i], d.scale);
}

// ---------------------------------------------------------------------------------------
// Row-vectorised pull collide-and-stream (nx even).  A warp covers 64 consecutive cells of
// one x-row, two per thread: every population is read as an aligned pair (half2 / float2 /
// double2) from its source row, and the +-1 shift along x of the populations with
// c_x != 0 is done with one warp shuffle (the lanes at the warp's ends fetch the missing
// neighbour with a scalar load, wrapping periodically at the row ends).  The nine source
// rows (y - c_y, z - c_z) are resolved once per thread.
template <class T, bool COUPLED>
__global__ void __launch_bounds__(256) k_collide_stream_rows(LatticeDesc d, const T* __restrict__ fin, T* __restrict__ fout,
                                                              const T* __restrict__ wall,
                                                              const typename Store<T>::F* __restrict__ Fcol,
                                                              typename Store<T>::F* __restrict__ Fprev,
                                                              typename Store<T>::U* __restrict__ u_out,
                                                              const uint8_t* __restrict__ phase,
                                                              const uint8_t* __restrict__ celltype, int coll) {
    using C = typename Store<T>::C;
    using FT = typename Store<T>::F;
    using UT = typename Store<T>::U;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // grid.x runs over blocks of rows (ny * nz can exceed the 65535 limit of grid.y)
    const int tx = blockIdx.y * blockDim.x + threadIdx.x;
    const int row = blockIdx.x * blockDim.y + threadIdx.y;
    if (row >= d.ny * d.nz) return;  // uniform per warp: a warp never spans two rows
    const int y = row % d.ny, z = row / d.ny;
    const int x0 = 2 * tx;
    const bool active = x0 < d.nx;
    const int64_t k0 = (int64_t)row * d.nx + x0;
    const bool wallrow = fd_wall_node(d, y);
    // ---- phase 1: issue every load of the cell pair before any shuffle or arithmetic, so
    // that all of them are in flight together (the shuffles would otherwise serialise them)
    C pa[Q], pb[Q], edge[Q];
    FT fpa[3], fpb[3], fca[3], fcb[3];
    int sface[3][3];
    if (wallrow) {
        const int64_t ws = wall_stride(d), wk = wall_index(d, y == 0 ? 0 : 1, active ? x0 : 0, z);
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            pa[i] = pb[i] = edge[i] = C(0);
            if (active) Pair<T>::load(wall + i * ws + wk, d.inv_scale, pa[i], pb[i]);
        }
    } else {
        int64_t srow[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                int ys = y - (a - 1), zs = z - (b - 1), face = -1;
                if (d.py) ys = (int)wrap_index(ys, d.ny);
                else if (ys < 0 || ys >= d.ny) face = ys < 0 ? 0 : 1;
                if (d.pz) zs = (int)wrap_index(zs, d.nz);
                else if (face < 0 && (zs < 0 || zs >= d.nz)) face = zs < 0 ? 2 : 3;
                sface[a][b] = face;
                srow[a][b] = face >= 0 ? -1 : ((int64_t)ys + (int64_t)d.ny * zs) * d.nx;
            }
        const int xl = x0 == 0 ? d.nx - 1 : x0 - 1;            // left neighbour of the pair
        const int xr = x0 + 2 >= d.nx ? x0 + 2 - d.nx : x0 + 2; // right neighbour of the pair
        const bool need_l = active && lane == 0;
        const bool need_r = active && (lane == 31 || x0 + 2 >= d.nx);
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const int a = cy(i) + 1, b = cz(i) + 1;
            pa[i] = pb[i] = edge[i] = C(0);
            if (srow[a][b] < 0) {
                // halfway bounce-back: the own node's opposite population, no shift in x
                if (active) Pair<T>::load(fin + opposite(i) * d.stride + k0, d.inv_scale, pa[i], pb[i]);
                continue;
            }
            const T* src = fin + i * d.stride + srow[a][b];
            if (active) Pair<T>::load(src + x0, d.inv_scale, pa[i], pb[i]);
            if (cx(i) == 1 && need_l) edge[i] = Store<T>::load(src + xl, d.inv_scale);
            if (cx(i) == -1 && need_r) edge[i] = Store<T>::load(src + xr, d.inv_scale);
        }
    }
    if (active) {
        for (int c = 0; c < 3; ++c) load2<FT>(Fcol + c * d.stride + k0, fca[c], fcb[c]);
        if (COUPLED && !wallrow) {
            if (Fprev) {
                for (int c = 0; c < 3; ++c) load2<FT>(Fprev + c * d.stride + k0, fpa[c], fpb[c]);
            } else {  // sparse force reset: the velocity field takes the body force only
                for (int c = 0; c < 3; ++c) fpa[c] = fpb[c] = (FT)d.body[c];
            }
        }
    }
    // ---- phase 2: assemble the gathered populations (x shifts through the warp)
    C f0[Q], f1[Q];
    if (wallrow) {
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            f0[i] = pa[i];
            f1[i] = pb[i];
        }
    } else {
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const int a = cy(i) + 1, b = cz(i) + 1;
            if (sface[a][b] >= 0) {
                const C mw = moving_wall_term<C>(d, i, sface[a][b]);
                f0[i] = pa[i] + mw;
                f1[i] = pb[i] + mw;
            } else if (cx(i) == 0) {
                f0[i] = pa[i];
                f1[i] = pb[i];
            } else if (cx(i) == 1) {  // src[x0 - 1], src[x0]
                const C left = __shfl_up_sync(FULL, pb[i], 1);
                f0[i] = lane == 0 ? edge[i] : left;
                f1[i] = pa[i];
            } else {  // src[x0 + 1], src[x0 + 2]
                const C right = __shfl_down_sync(FULL, pa[i], 1);
                f0[i] = pb[i];
                f1[i] = (lane == 31 || x0 + 2 >= d.nx) ? edge[i] : right;
            }
        }
    }
    if (!active) return;
    int ct0 = BIB_CELL_FLUID, ct1 = BIB_CELL_FLUID;
    if (d.has_types) {
        ct0 = celltype[k0];
        ct1 = celltype[k0 + 1];
    }
    if (COUPLED) {
        C u0[3], u1[3];
        if (wallrow) {
            const int side = y == 0 ? 0 : 1;
            for (int c = 0; c < 3; ++c) u0[c] = u1[c] = (C)d.wall_u[side][c];
        } else {
            C Fa[3] = {(C)fpa[0], (C)fpa[1], (C)fpa[2]}, Fb[3] = {(C)fpb[0], (C)fpb[1], (C)fpb[2]};
            velocity_with_force(f0, Fa, u0);
            velocity_with_force(f1, Fb, u1);
        }
        if (ct0 != BIB_CELL_FLUID) u0[0] = u0[1] = u0[2] = C(0);
        if (ct1 != BIB_CELL_FLUID) u1[0] = u1[1] = u1[2] = C(0);
        store_u<UT>(u_out, k0, (UT)u0[0], (UT)u0[1], (UT)u0[2]);
        store_u<UT>(u_out, k0 + 1, (UT)u1[0], (UT)u1[1], (UT)u1[2]);
        if (Fprev)
            for (int c = 0; c < 3; ++c) store2<FT>(Fprev + c * d.stride + k0, (FT)d.body[c], (FT)d.body[c]);
    }
    C Fa[3] = {(C)fca[0], (C)fca[1], (C)fca[2]}, Fb[3] = {(C)fcb[0], (C)fcb[1], (C)fcb[2]};
    C om0 = (C)d.omega, om1 = (C)d.omega, omm = C(0);
    if (coll == BIB_COLLISION_BGK_GUO_VOF) {
        om0 = om1 = (C)d.omega_c0;
        if (d.use_phase) {
            if (phase[k0]) om0 = (C)d.omega_c1;
            if (phase[k0 + 1]) om1 = (C)d.omega_c1;
        }
    } else if (coll == BIB_COLLISION_TRT) {
        omm = C(1) / ((C)d.trt_magic / (C(1) / om0 - C(0.5)) + C(0.5));
    }
    auto collide_one = [&](C* f, const C* Fx, C om) {
        if (coll == BIB_COLLISION_BGK_GUO_VOF) collide_unscaled<C, BIB_COLLISION_BGK_GUO_VOF>(f, Fx, om, C(0));
        else if (coll == BIB_COLLISION_BGK) collide_unscaled<C, BIB_COLLISION_BGK>(f, Fx, om, C(0));
        else collide_unscaled<C, BIB_COLLISION_TRT>(f, Fx, om, omm);
    };
    // BounceBack nodes swap their incoming populations, NoDynamics nodes keep them
    if (ct0 == BIB_CELL_FLUID) collide_one(f0, Fa, om0);
    else if (ct0 == BIB_CELL_BOUNCE_BACK) bounce_back_cell(f0);
    if (ct1 == BIB_CELL_FLUID) collide_one(f1, Fb, om1);
    else if (ct1 == BIB_CELL_BOUNCE_BACK) bounce_back_cell(f1);
#pragma unroll
    for (int i = 0; i < Q; ++i) Pair<T>::store(fout + i * d.stride + k0, f0[i], f1[i], d.scale);
}

// PlaneFdBoundaryFunctional3D::processCell on the y walls after collide-and-stream,
// src/boundaryCondition/finiteDifferenceBoundaryProcessor3D.hh:68-115: density from the
// known populations (VelocityDirichletBoundaryDynamics::computeRhoBar,
// boundaryDynamics.hh:631-663), one-sided normal velocity derivative
// (finiteDifference3D.h:67-82; tangential derivatives vanish for a uniform wall
// velocity), regularised reconstruction of all 19 populations into the wall buffer.
template <class T>
__device__ __forceinline__ void fd_wall_cell(const LatticeDesc& d, const T* __restrict__ f, T* __restrict__ wall,
                                             const typename Store<T>::F* __restrict__ F, int x, int z, int side);

// GuoRigidWallBoundaryFunctional::process with depth 2 (fsi/GuoBoundaryCondition.hh:133-187),
// one thread per wall node after collide-and-stream: the post-streaming states of the two fluid
// nodes along the node's lattice vector give density, momentum and non-equilibrium parts; the
// node's new state, the equilibrium of the extrapolated wall momentum (0 for a NoDynamics node)
// plus the extrapolated non-equilibrium part, is scattered into the post-collision slots it
// gathers from.  Each slot f*_i(x) is read by the node x + c_i alone, and no wall node's fluid
// nodes are wall nodes (checked on the host), so the threads never touch each other's data.
template <class T>
__global__ void __launch_bounds__(128) k_guo_walls(LatticeDesc d, T* __restrict__ f, const T* __restrict__ wall,
                                                    const GuoNode* __restrict__ nodes, int n) {
    using C = typename Store<T>::C;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const GuoNode w = nodes[g];
    C fc[2][Q], rb[2], j[2][3], fneq[2][Q];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int xs = (int)wrap_index(w.x + (m + 1) * cx(w.dir), d.nx);
        const int ys = (int)wrap_index(w.y + (m + 1) * cy(w.dir), d.ny);
        const int zs = (int)wrap_index(w.z + (m + 1) * cz(w.dir), d.nz);
        gather<T>(d, f, wall, xs, ys, zs, xs + (int64_t)d.nx * (ys + (int64_t)d.ny * zs), fc[m]);
        rho_bar_j<C>(fc[m], rb[m], j[m]);
        const C jsq = j[m][0] * j[m][0] + j[m][1] * j[m][1] + j[m][2] * j[m][2];
        const C invRho = C(1) / (rb[m] + C(1));
#pragma unroll
        for (int i = 0; i < Q; ++i) fneq[m][i] = fc[m][i] - bgk_equilibrium<C>(i, rb[m], invRho, j[m], jsq);
    }
    const C rbw = rb[0], dl = (C)w.delta;
    C wj[3], jw[3], fw[Q];
    for (int c = 0; c < 3; ++c) wj[c] = (rbw + C(1)) * (C)w.u[c];
    if (dl < C(0.75)) {
        for (int c = 0; c < 3; ++c)
            jw[c] = wj[c] + (dl - C(1)) * j[0][c] + (C(1) - dl) / (C(1) + dl) * (C(2) * wj[c] + (dl - C(1)) * j[1][c]);
#pragma unroll
        for (int i = 0; i < Q; ++i) fw[i] = dl * fneq[0][i] + (C(1) - dl) * fneq[1][i];
    } else {
        for (int c = 0; c < 3; ++c) jw[c] = C(1) / dl * (wj[c] + (dl - C(1)) * j[0][c]);
#pragma unroll
        for (int i = 0; i < Q; ++i) fw[i] = fneq[0][i];
    }
    const C jsq = jw[0] * jw[0] + jw[1] * jw[1] + jw[2] * jw[2];
    const C invRho = C(1) / (rbw + C(1));
    const int64_t k = w.x + (int64_t)d.nx * (w.y + (int64_t)d.ny * w.z);
#pragma unroll
    for (int i = 0; i < Q; ++i)
        scatter_canonical<T>(d, f, const_cast<T*>(wall), i, w.x, w.y, w.z, k,
                             (w.nodyn ? C(0) : bgk_equilibrium<C>(i, rbw, invRho, jw, jsq)) + fw[i]);
}

template <class T>
__global__ void k_fd_walls(LatticeDesc d, const T* __restrict__ f, T* __restrict__ wall,
                           const typename Store<T>::F* __restrict__ F) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= d.nx) return;
    fd_wall_cell<T>(d, f, wall, F, x, blockIdx.y, blockIdx.z);
}

// Batched: grid.z = 2 sides x lattices; each lattice's view of the state after the swap.
template <class T>
__global__ void k_fd_walls_batch(const CollideView* __restrict__ views) {
    const CollideView& V = views[blockIdx.z >> 1];
    const int x = blockIdx.x * blockDim.x + threadIdx.x, z = blockIdx.y;
    if (!V.d.fd_walls || x >= V.d.nx || z >= V.d.nz) return;
    fd_wall_cell<T>(V.d, static_cast<const T*>(V.fin), static_cast<T*>(const_cast<void*>(V.wall)),
                    static_cast<const typename Store<T>::F*>(V.Fprev), x, z, blockIdx.z & 1);
}

template <class T>
__device__ __forceinline__ void fd_wall_cell(const LatticeDesc& d, const T* __restrict__ f, T* __restrict__ wall,
                                             const typename Store<T>::F* __restrict__ F, int x, int z, int side) {
    using C = typename Store<T>::C;
    const int y = side == 0 ? 0 : d.ny - 1;
    const int orientation = side == 0 ? -1 : 1;
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    const int y1 = y - orientation;
    const int64_t k1 = x + (int64_t)d.nx * (y1 + (int64_t)d.ny * z);
    C fc[Q], f1[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        int face;
        const int64_t s = source_cell(d, i, x, y, z, face);
        fc[i] = s >= 0 ? Store<T>::load(f + i * d.stride + s, d.inv_scale) : C(0);  // unknown ones are not used
    }
    gather<T>(d, f, wall, x, y1, z, k1, f1);
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
    const int64_t wk = wall_index(d, side, x, z), ws = wall_stride(d);
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
        Store<T>::store(wall + i * ws + wk, bgk_equilibrium<C>(i, rhoBar, invRho, j, jSqr) + fneq, d.scale);
    }
}

// computeVelocity of the current state with the current external force F (wall nodes
// give the wall velocity); OT = double for the host export, the compute type otherwise.
template <class T, class OT>
__global__ void k_velocity(LatticeDesc d, const T* __restrict__ f, const T* __restrict__ wall,
                           const typename Store<T>::F* __restrict__ F, OT* __restrict__ u, int64_t cstride,
                           int64_t kstride, const uint8_t* __restrict__ celltype) {
    using C = typename Store<T>::C;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= d.nx) return;
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    C uc[3];
    if (d.has_types && celltype[k] != BIB_CELL_FLUID) {  // BounceBack / NoDynamics: zero velocity
        uc[0] = uc[1] = uc[2] = C(0);
    } else if (fd_wall_node(d, y)) {
        const int side = y == 0 ? 0 : 1;
        for (int a = 0; a < 3; ++a) uc[a] = (C)d.wall_u[side][a];
    } else {
        C fc[Q];
        gather<T>(d, f, wall, x, y, z, k, fc);
        C Fc[3] = {(C)F[k], (C)F[d.stride + k], (C)F[2 * d.stride + k]};
        velocity_with_force(fc, Fc, uc);
    }
    for (int a = 0; a < 3; ++a) u[a * cstride + k * kstride] = (OT)uc[a];
    if (kstride == 4) u[k * 4 + 3] = OT(0.0f);
}

// iniCellAtEquilibrium, src/core/cell.hh:124-132, in the storage's compute type (FP64 for FP64
// storage; FP32 otherwise: the FP64 pipe of this part would make the 19 equilibria per cell
// slower than reading the host velocity field over the CPU-GPU link).
template <class T>
__global__ void k_init_eq(LatticeDesc d, T* __restrict__ f, T* __restrict__ wall, const double* __restrict__ rho,
                          const double* __restrict__ u) {
    using C = typename Store<T>::C;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= d.nx) return;
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    const double r = rho ? rho[k] : 1.0;
    const C j[3] = {(C)(u[k] * r), (C)(u[d.n + k] * r), (C)(u[2 * d.n + k] * r)};
    const C jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    const double rb = r - 1.0;
    const C rhoBar = (C)rb, invRho = (C)(1.0 / (rb + 1.0));
#pragma unroll
    for (int i = 0; i < Q; ++i) scatter_canonical<T>(d, f, wall, i, x, y, z, k, bgk_equilibrium<C>(i, rhoBar, invRho, j, jSqr));
}

// Import / export of the planes z0 .. z0 + gridDim.z - 1 from / to a buffer holding, per
// population, `pitch` cells that start with the first cell of plane z0.
template <class T>
__global__ void k_import(LatticeDesc d, T* __restrict__ f, T* __restrict__ wall, const double* __restrict__ src, int z0,
                         int64_t pitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = z0 + (int)blockIdx.z;
    if (x >= d.nx) return;
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    const int64_t j = k - (int64_t)z0 * d.nx * d.ny;
#pragma unroll
    for (int i = 0; i < Q; ++i) scatter_canonical<T>(d, f, wall, i, x, y, z, k, src[i * pitch + j]);
}

template <class T>
__global__ void k_export(LatticeDesc d, const T* __restrict__ f, const T* __restrict__ wall, double* __restrict__ dst,
                         int z0, int64_t pitch) {
    using C = typename Store<T>::C;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = z0 + (int)blockIdx.z;
    if (x >= d.nx) return;
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    const int64_t j = k - (int64_t)z0 * d.nx * d.ny;
    C fc[Q];
    gather<T>(d, f, wall, x, y, z, k, fc);
    for (int i = 0; i < Q; ++i) dst[i * pitch + j] = (double)fc[i];
}

// Import / export of the cells w0 .. w0 + count - 1 of the cell-major wire order of Palabos
// (BlockLattice3D static content, blockLattice3D.hh:644-689: x slowest, z fastest; `per` = 23
// doubles per cell: 19 f-bar, the force, the phase) and of CoProcessor3D (coProcessor3D.h:84-91:
// the same order, `per` = 19 populations only).  `src` / `dst` hold cell w0 first.  Consecutive
// threads take consecutive cells, so a warp reads or writes one contiguous run of the buffer; the
// strided lattice accesses merge in L2.
template <class T>
__global__ void k_import_aos(LatticeDesc d, T* __restrict__ f, T* __restrict__ wall, typename Store<T>::F* __restrict__ F,
                             uint8_t* __restrict__ phase, const double* __restrict__ src, int per, int64_t w0,
                             int64_t count) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t w = w0 + t, r = w / d.nz;
    const int z = (int)(w - r * d.nz), y = (int)(r % d.ny), x = (int)(r / d.ny);
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    const double* s = src + per * t;
#pragma unroll
    for (int i = 0; i < Q; ++i) scatter_canonical<T>(d, f, wall, i, x, y, z, k, s[i]);
    if (per == Q + 4) {
        for (int a = 0; a < 3; ++a) F[a * d.stride + k] = (typename Store<T>::F)s[Q + a];
        if (phase) phase[k] = s[Q + 3] >= 0.5 ? 1 : 0;
    }
}

template <class T>
__global__ void k_export_aos(LatticeDesc d, const T* __restrict__ f, const T* __restrict__ wall,
                             const typename Store<T>::F* __restrict__ F, const uint8_t* __restrict__ phase,
                             double* __restrict__ dst, int per, int64_t w0, int64_t count) {
    using C = typename Store<T>::C;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t w = w0 + t, r = w / d.nz;
    const int z = (int)(w - r * d.nz), y = (int)(r % d.ny), x = (int)(r / d.ny);
    const int64_t k = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
    C fc[Q];
    gather<T>(d, f, wall, x, y, z, k, fc);
    double* o = dst + per * t;
#pragma unroll
    for (int i = 0; i < Q; ++i) o[i] = (double)fc[i];
    if (per == Q + 4) {
        for (int a = 0; a < 3; ++a) o[Q + a] = (double)F[a * d.stride + k];
        o[Q + 3] = phase && phase[k] ? 1.0 : 0.0;
    }
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

inline int row_block(const LatticeDesc& d) { return d.nx >= 256 ? 256 : (d.nx >= 128 ? 128 : (d.nx >= 64 ? 64 : 32)); }
inline dim3 row_grid(const LatticeDesc& d, int bx) { return dim3((d.nx + bx - 1) / bx, d.ny, d.nz); }
inline unsigned lin_grid(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

template <class T>
void collide_stream_t(const Lattice& L, Coupling mode, cudaStream_t s) {
    using FT = typename Store<T>::F;
    if (L.collide_kernel != BIB_KERNEL_ROWS && launch_collide_stream_staged(L, mode, s)) return;
    const bool coupled = mode != Coupling::kNone;
    // the previous force, read for the velocity and reset (dense coupling only)
    FT* Fprev = mode == Coupling::kDense ? (FT*)L.F[L.fe] : nullptr;
    if (L.d.nx % 2 == 0) {
        const int pairs = L.d.nx / 2;
        const int bx = std::min(256, (pairs + 31) / 32 * 32);
        const int by = std::max(1, 256 / bx);
        const int rows = L.d.ny * L.d.nz;
        dim3 grid((rows + by - 1) / by, (pairs + bx - 1) / bx);
        dim3 block(bx, by);
        const T* fin = (const T*)L.f[L.cur];
        T* fout = (T*)L.f[1 - L.cur];
        if (coupled)
            k_collide_stream_rows<T, true><<<grid, block, 0, s>>>(L.d, fin, fout, (const T*)L.wall, (const FT*)L.F[1 - L.fe],
                                                                  Fprev, (typename Store<T>::U*)L.u, L.phase, L.celltype, L.d.collision);
        else
            k_collide_stream_rows<T, false><<<grid, block, 0, s>>>(L.d, fin, fout, (const T*)L.wall, (const FT*)L.F[L.fe],
                                                                   nullptr, nullptr, L.phase, L.celltype, L.d.collision);
        return;
    }
    const int bx = row_block(L.d);
    const T* fin = (const T*)L.f[L.cur];
    T* fout = (T*)L.f[1 - L.cur];
    const T* wall = (const T*)L.wall;
    if (coupled) {
        k_collide_stream<T, true><<<row_grid(L.d, bx), bx, 0, s>>>(L.d, fin, fout, wall, (const FT*)L.F[1 - L.fe],
                                                                    Fprev, (typename Store<T>::U*)L.u, L.phase, L.celltype, L.d.collision);
    } else {
        k_collide_stream<T, false><<<row_grid(L.d, bx), bx, 0, s>>>(L.d, fin, fout, wall, (const FT*)L.F[L.fe], nullptr,
                                                                     nullptr, L.phase, L.celltype, L.d.collision);
    }
}

template <class T>
void fd_walls_batch_t(const BatchLaunch& B, cudaStream_t s) {
    const int bx = B.nx_max >= 128 ? 128 : 64;
    dim3 g((B.nx_max + bx - 1) / bx, B.nz_max, 2 * B.n);
    k_fd_walls_batch<T><<<g, bx, 0, s>>>(B.wviews);
}

template <class T>
void fd_walls_t(const Lattice& L, int buf, int fbuf, cudaStream_t s) {
    using FT = typename Store<T>::F;
    const int bx = row_block(L.d);
    dim3 g((L.d.nx + bx - 1) / bx, L.d.nz, 2);
    k_fd_walls<T><<<g, bx, 0, s>>>(L.d, (const T*)L.f[buf], (T*)L.wall, (const FT*)L.F[fbuf]);
}

#define BIB_DISPATCH(storage, FN, ...)                          \
    do {                                                       \
        if ((storage) == BIB_STORAGE_F64) FN<double>(__VA_ARGS__); \
        else if ((storage) == BIB_STORAGE_F32) FN<float>(__VA_ARGS__); \
        else FN<__half>(__VA_ARGS__);                          \
    } while (0)

template <class T>
void velocity_field_t(const Lattice& L, cudaStream_t s) {
    using FT = typename Store<T>::F;
    using UT = typename Store<T>::U;
    const int bx = row_block(L.d);
    k_velocity<T, UT><<<row_grid(L.d, bx), bx, 0, s>>>(L.d, (const T*)L.f[L.cur], (const T*)L.wall, (const FT*)L.F[L.fe],
                                                        (UT*)L.u, 1, 4, L.celltype);
}

template <class T>
void velocity_export_t(const Lattice& L, double* u, cudaStream_t s) {
    using FT = typename Store<T>::F;
    const int bx = row_block(L.d);
    k_velocity<T, double><<<row_grid(L.d, bx), bx, 0, s>>>(L.d, (const T*)L.f[L.cur], (const T*)L.wall,
                                                            (const FT*)L.F[L.fe], u, L.d.n, 1, L.celltype);
}

template <class T>
void init_eq_t(const Lattice& L, const double* rho, const double* u, cudaStream_t s) {
    const int bx = row_block(L.d);
    k_init_eq<T><<<row_grid(L.d, bx), bx, 0, s>>>(L.d, (T*)L.f[L.cur], (T*)L.wall, rho, u);
}

template <class T>
void import_t(const Lattice& L, const double* src, int z0, int nzc, int64_t pitch, cudaStream_t s) {
    const int bx = row_block(L.d);
    dim3 g((L.d.nx + bx - 1) / bx, L.d.ny, nzc);
    k_import<T><<<g, bx, 0, s>>>(L.d, (T*)L.f[L.cur], (T*)L.wall, src, z0, pitch);
}

template <class T>
void export_t(const Lattice& L, double* dst, int z0, int nzc, int64_t pitch, cudaStream_t s) {
    const int bx = row_block(L.d);
    dim3 g((L.d.nx + bx - 1) / bx, L.d.ny, nzc);
    k_export<T><<<g, bx, 0, s>>>(L.d, (const T*)L.f[L.cur], (const T*)L.wall, dst, z0, pitch);
}

template <class T>
void import_aos_t(const Lattice& L, const double* src, int per, int64_t w0, int64_t count, cudaStream_t s) {
    using FT = typename Store<T>::F;
    k_import_aos<T><<<lin_grid(count, 256), 256, 0, s>>>(L.d, (T*)L.f[L.cur], (T*)L.wall, (FT*)L.F[L.fe], L.phase, src,
                                                         per, w0, count);
}

template <class T>
void export_aos_t(const Lattice& L, double* dst, int per, int64_t w0, int64_t count, cudaStream_t s) {
    using FT = typename Store<T>::F;
    k_export_aos<T><<<lin_grid(count, 256), 256, 0, s>>>(L.d, (const T*)L.f[L.cur], (const T*)L.wall,
                                                         (const FT*)L.F[L.fe], L.phase, dst, per, w0, count);
}

template <class T>
void nan_scan_t(const Lattice& L, int* flag, cudaStream_t s) {
    k_nan_scan<T><<<lin_grid(L.d.n, 256), 256, 0, s>>>(L.d, (const T*)L.f[L.cur], flag);
}

}  // namespace

void launch_collide_stream(const Lattice& L, Coupling mode, cudaStream_t s) {
    BIB_DISPATCH(L.storage, collide_stream_t, L, mode, s);
}

void launch_fd_walls_batch(const BatchLaunch& B, cudaStream_t s) {
    if (!B.any_fd || B.n == 0) return;
    BIB_DISPATCH(B.storage, fd_walls_batch_t, B, s);
}

template <class T>
void guo_walls_t(const Lattice& L, int buf, cudaStream_t s) {
    k_guo_walls<T><<<(L.nguo + 127) / 128, 128, 0, s>>>(L.d, (T*)L.f[buf], (const T*)L.wall, L.guo, L.nguo);
}

// The wall processors after a collide-and-stream: finite-difference velocity walls, then the
// second-order rigid walls (the latter integrated at processor level 1, after the former)
void launch_fd_walls(const Lattice& L, int buf, int fbuf, cudaStream_t s) {
    if (L.d.fd_walls) BIB_DISPATCH(L.storage, fd_walls_t, L, buf, fbuf, s);
    if (L.nguo > 0) BIB_DISPATCH(L.storage, guo_walls_t, L, buf, s);
}

namespace {
__global__ void __launch_bounds__(256) k_copy_f64(double* __restrict__ dst, const double* __restrict__ src, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) dst[i] = src[i];
}
}  // namespace

void launch_copy_f64(double* dst, const double* src, size_t n, cudaStream_t s) {
    if (n == 0) return;
    const unsigned g = (unsigned)std::min<size_t>((n + 255) / 256, 1024);
    k_copy_f64<<<g, 256, 0, s>>>(dst, src, n);
}

void launch_velocity_field(const Lattice& L, cudaStream_t s) { BIB_DISPATCH(L.storage, velocity_field_t, L, s); }

void launch_velocity_export(const Lattice& L, double* u, cudaStream_t s) {
    BIB_DISPATCH(L.storage, velocity_export_t, L, u, s);
}

void launch_init_equilibrium(const Lattice& L, const double* rho, const double* u, cudaStream_t s) {
    BIB_DISPATCH(L.storage, init_eq_t, L, rho, u, s);
}

void launch_import_planes(const Lattice& L, const double* src, int z0, int nzc, int64_t pitch, cudaStream_t s) {
    BIB_DISPATCH(L.storage, import_t, L, src, z0, nzc, pitch, s);
}

void launch_export_planes(const Lattice& L, double* dst, int z0, int nzc, int64_t pitch, cudaStream_t s) {
    BIB_DISPATCH(L.storage, export_t, L, dst, z0, nzc, pitch, s);
}

void launch_import_aos(const Lattice& L, const double* src, int per, int64_t w0, int64_t count, cudaStream_t s) {
    if (count > 0) BIB_DISPATCH(L.storage, import_aos_t, L, src, per, w0, count, s);
}

void launch_export_aos(const Lattice& L, double* dst, int per, int64_t w0, int64_t count, cudaStream_t s) {
    if (count > 0) BIB_DISPATCH(L.storage, export_aos_t, L, dst, per, w0, count, s);
}

void launch_force_import(const Lattice& L, int buf, const double* src, cudaStream_t s) {
    const unsigned g = lin_grid(L.d.n, 256);
    if (L.storage == BIB_STORAGE_F64) k_force_import<double><<<g, 256, 0, s>>>(L.d, (double*)L.F[buf], src);
    else k_force_import<float><<<g, 256, 0, s>>>(L.d, (float*)L.F[buf], src);
}

void launch_force_export(const Lattice& L, int buf, double* dst, cudaStream_t s) {
    const unsigned g = lin_grid(L.d.n, 256);
    if (L.storage == BIB_STORAGE_F64) k_force_export<double><<<g, 256, 0, s>>>(L.d, (const double*)L.F[buf], dst);
    else k_force_export<float><<<g, 256, 0, s>>>(L.d, (const float*)L.F[buf], dst);
}

void launch_force_fill(const Lattice& L, int buf, cudaStream_t s) {
    const size_t fsz = L.storage == BIB_STORAGE_F64 ? sizeof(double) : sizeof(float);
    if (L.d.body[0] == 0.0 && L.d.body[1] == 0.0 && L.d.body[2] == 0.0) {
        cudaMemsetAsync(L.F[buf], 0, 3 * L.d.stride * fsz, s);
        return;
    }
    const unsigned g = lin_grid(L.d.stride, 256);
    if (L.storage == BIB_STORAGE_F64) k_force_fill<double><<<g, 256, 0, s>>>(L.d, (double*)L.F[buf]);
    else k_force_fill<float><<<g, 256, 0, s>>>(L.d, (float*)L.F[buf]);
}

void launch_phase_import(const Lattice& L, const double* src, cudaStream_t s) {
    k_phase_import<<<lin_grid(L.d.n, 256), 256, 0, s>>>(L.d, L.phase, src);
}

void launch_nan_scan(const Lattice& L, int* flag, cudaStream_t s) { BIB_DISPATCH(L.storage, nan_scan_t, L, flag, s); }

}  // namespace bib
