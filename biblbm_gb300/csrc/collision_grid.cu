// The reference's collision grid and the rigid-body growth of the initial distribution.
//
// Collision grid (fsi/CollisionForces.h:63-199, fsi/Grid.hh:28-99, with the node set of
// ImmersedBoundaryDynamics_forces.hh:330-375): the box [x0 - 1/2, x1 + 1/2 - eps] per axis is cut
// into ~unit cells with one envelope layer; vertices inside the box enlarged by the cutoff join
// the cell they fall in, in vertex order.  Every bulk cell pairs its vertices among themselves and
// with those of 7 of its 13 forward neighbours; on periodic axes the first and last bulk layers are
// paired too.  Pairs in cells at the other 6 forward offsets are never examined: this is the
// reference's search, kept as a parity mode beside the every-pair search of ib_kernels.cu.
//
// Each vertex is one thread: it enumerates the pair events that touch it in the order of the
// reference's loops (cells in (x, y, z) order, vertices in order, the 7 neighbours in order, then
// the periodic layer passes) and accumulates them one by one, rounding each product and sum alone
// (no contraction), so the forces equal the reference's sequential accumulation bit for bit.
//
// Growth (progs/common/create_particles.h:105-161, fsi/RigidParticle.hh): rigid copies of shapes,
// rescaled every few iterations, pushed apart by those collision forces and a pipe wall, moved as
// rigid bodies.  One CTA per particle: the force and torque sums in vertex order, the integration
// and the vertex regeneration.
#include <cub/device/device_radix_sort.cuh>

#include <cfloat>
#include <cmath>

#include "bib_internal.h"

namespace bib {

namespace {

// Products and sums rounded one at a time, as the reference's build evaluates them.
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// SpringPotential::operator() / MorsePotential (fsi/Potentials.h:29-71)
__device__ __forceinline__ double grid_potential(const PotentialDev& p, double d) {
    if (p.kind == BIB_POTENTIAL_SPRING) return mul(sub(p.r0, d), p.strength);
    if (p.kind == BIB_POTENTIAL_MORSE) {
        if (d < 0) d = 0.0;
        const double x = exp(mul(p.beta, sub(p.r0, d)));
        return mul(mul(mul(mul(2.0, p.beta), p.strength), x), sub(x, 1.0));
    }
    return 0.0;
}

struct GridArgs {
    RefGrid g;
    PotentialDev pot;
    double c2;  // cutoff squared
    // FP32 pre-test: a pair whose FP32 distance (positions rounded to FP32, the minimum image taken
    // in FP32) exceeds sqrt(pre_c2) is beyond the cutoff for certain (the margin covers the
    // rounding), so the exact FP64 test, which alone decides, is skipped.  pre_c2 <= 0: off.
    float pre_c2;
    float Lf[3], Linvf[3];
    const float4* posf;
    const double* pos;
    const int* owner;
    const uint32_t* keys;  // sorted cell keys
    const uint32_t* ids;   // vertex of each sorted slot
    const int* start;
    const int* end;
};

// Arithmetic1D::min_mod_diff (fsi/Periodicity.h:27-35, 96-99)
__device__ __forceinline__ double grid_diff(const RefGrid& g, int a, double x, double y) {
    const double d = sub(x, y);
    if (!g.per[a]) return d;
    return sub(d, mul(floor(add(mul(d, g.Linv[a]), 0.5)), g.L[a]));
}

// handle_collision(node, node2) (CollisionForces.h:187-199) seen from one of its vertices:
// `first` when the vertex is `node` (force += df), else it is `node2` (force -= df).
__device__ __forceinline__ void grid_event(const GridArgs& A, int a, const double* xa, const float4& xaf, int b,
                                           bool first, double* f) {
    if (A.owner[a] == A.owner[b]) return;
    if (A.pre_c2 > 0.0f) {
        const float4 q = A.posf[b];
        float e[3] = {q.x - xaf.x, q.y - xaf.y, q.z - xaf.z};
        for (int d = 0; d < 3; ++d)
            if (A.g.per[d]) e[d] -= A.Lf[d] * rintf(e[d] * A.Linvf[d]);
        if (e[0] * e[0] + e[1] * e[1] + e[2] * e[2] > A.pre_c2) return;
    }
    const double* xb = A.pos + 3LL * b;
    double dr[3];
    for (int d = 0; d < 3; ++d) dr[d] = first ? grid_diff(A.g, d, xb[d], xa[d]) : grid_diff(A.g, d, xa[d], xb[d]);
    const double dsq = add(add(mul(dr[0], dr[0]), mul(dr[1], dr[1])), mul(dr[2], dr[2]));
    if (!(dsq <= A.c2)) return;
    const double dist = __dsqrt_rn(dsq);
    const double s = dvd(-grid_potential(A.pot, dist), dist);
    for (int d = 0; d < 3; ++d) f[d] = first ? add(f[d], mul(s, dr[d])) : sub(f[d], mul(s, dr[d]));
}

__device__ __forceinline__ int grid_cell(const RefGrid& g, int i, int j, int k) { return k + g.nc[2] * (j + g.nc[1] * i); }

// collide_all_in_cells(c1, c2) (CollisionForces.h:178-184): the events of the vertex at slot s
__device__ void grid_all_in_cells(const GridArgs& A, int c1, int c2, int c, int s, int a, const double* xa,
                                  const float4& xaf, double* f) {
    if (c1 == c2) {
        for (int l = A.start[c1]; l < A.end[c1]; ++l) {
            if (l == s) {
                for (int m = A.start[c2]; m < A.end[c2]; ++m)
                    if (m != s) grid_event(A, a, xa, xaf, (int)A.ids[m], true, f);
            } else {
                grid_event(A, a, xa, xaf, (int)A.ids[l], false, f);
            }
        }
    } else if (c == c1) {
        for (int m = A.start[c2]; m < A.end[c2]; ++m) grid_event(A, a, xa, xaf, (int)A.ids[m], true, f);
    } else if (c == c2) {
        for (int l = A.start[c1]; l < A.end[c1]; ++l) grid_event(A, a, xa, xaf, (int)A.ids[l], false, f);
    }
}

// Key of a vertex: its cell (Grid::insert, Grid.hh:74-82) when it lies strictly inside the box
// enlarged by the cutoff (geo::Rect::contains), else the sentinel ncell.
__global__ void __launch_bounds__(128) k_grid_keys(RefGrid g, int nvert, const double* __restrict__ pos,
                                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ ids,
                                                    float4* __restrict__ posf) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvert) return;
    const double* x = pos + 3LL * v;
    posf[v] = make_float4((float)x[0], (float)x[1], (float)x[2], 0.0f);
    uint32_t key = (uint32_t)g.ncell;
    bool in = true;
    int ci[3];
    for (int a = 0; a < 3; ++a) {
        in = in && x[a] > g.lo[a] && x[a] < g.hi[a];
        const double t = floor(dvd(sub(x[a], g.g0[a]), g.cs[a]));
        ci[a] = (t >= 0.0 && t < (double)g.nc[a]) ? (int)t : -1;
        in = in && ci[a] >= 0;
    }
    if (in) key = (uint32_t)grid_cell(g, ci[0], ci[1], ci[2]);
    keys[v] = key;
    ids[v] = (uint32_t)v;
}

__global__ void __launch_bounds__(128) k_grid_clear(int nvert, const uint32_t* __restrict__ prev_keys, int* start,
                                                     int* end) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nvert) return;
    start[prev_keys[s]] = 0;
    end[prev_keys[s]] = 0;
}

__global__ void __launch_bounds__(128) k_grid_bounds(int nvert, const uint32_t* __restrict__ keys, int* start,
                                                      int* end) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nvert) return;
    const uint32_t k = keys[s];
    if (s == 0 || keys[s - 1] != k) start[k] = s;
    if (s == nvert - 1 || keys[s + 1] != k) end[k] = s + 1;
}

// One thread per sorted slot.  ZERO: the forces start at zero (set_forces_to_zero) and vertices
// outside the grid are written too; else the events are added to the forces in place.  wall (y0,
// z0, radius; radius <= 0: none) adds compute_wall_collision_forces (CollisionForces.h:166-184).
template <bool ZERO>
__global__ void __launch_bounds__(128) k_grid_forces(GridArgs A, double wy0, double wz0, double wr,
                                                      double* __restrict__ force) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int nvert = A.g.nvert;
    if (s >= nvert) return;
    const int a = (int)A.ids[s];
    const int c = (int)A.keys[s];
    double* fo = force + 3LL * a;
    double f[3];
    for (int d = 0; d < 3; ++d) f[d] = ZERO ? 0.0 : fo[d];
    if (c >= A.g.ncell) {
        if (ZERO)
            for (int d = 0; d < 3; ++d) fo[d] = 0.0;
        return;
    }
    const RefGrid& g = A.g;
    const double xa[3] = {A.pos[3LL * a], A.pos[3LL * a + 1], A.pos[3LL * a + 2]};
    const float4 xaf = A.posf[a];
    const int k = c % g.nc[2], j = (c / g.nc[2]) % g.nc[1], i = c / (g.nc[2] * g.nc[1]);
    const int x0 = 1, x1 = g.nc[0] - 2, y0 = 1, y1 = g.nc[1] - 2, z0 = 1, z1 = g.nc[2] - 2;
    auto bulk = [&](int p, int q, int r) { return p >= x0 && p <= x1 && q >= y0 && q <= y1 && r >= z0 && r <= z1; };
    // events of earlier cells whose neighbour this cell is, in increasing cell order
    const int pre[7][3] = {{1, 1, 1}, {1, 1, 0}, {1, 0, 1}, {1, 0, 0}, {0, 1, 1}, {0, 1, 0}, {0, 0, 1}};
    for (int n = 0; n < 7; ++n) {
        const int p = i - pre[n][0], q = j - pre[n][1], r = k - pre[n][2];
        if (!bulk(p, q, r)) continue;
        const int cp = grid_cell(g, p, q, r);
        for (int l = A.start[cp]; l < A.end[cp]; ++l) grid_event(A, a, xa, xaf, (int)A.ids[l], false, f);
    }
    if (bulk(i, j, k)) {
        for (int l = A.start[c]; l < s; ++l) grid_event(A, a, xa, xaf, (int)A.ids[l], false, f);
        for (int m = s + 1; m < A.end[c]; ++m) grid_event(A, a, xa, xaf, (int)A.ids[m], true, f);
        const int nb[7][3] = {{0, 1, 0}, {0, 1, 1}, {0, 0, 1}, {1, 0, 0}, {1, 1, 0}, {1, 1, 1}, {1, 0, 1}};
        for (int n = 0; n < 7; ++n) {
            const int cn = grid_cell(g, i + nb[n][0], j + nb[n][1], k + nb[n][2]);
            for (int m = A.start[cn]; m < A.end[cn]; ++m) grid_event(A, a, xa, xaf, (int)A.ids[m], true, f);
        }
        // the first and last bulk layers of periodic axes (CollisionForces.h:119-163)
        if (g.per[0] && (i == x0 || i == x1)) grid_all_in_cells(A, grid_cell(g, x0, j, k), grid_cell(g, x1, j, k), c, s, a, xa, xaf, f);
        if (g.per[1] && (j == y0 || j == y1)) grid_all_in_cells(A, grid_cell(g, i, y0, k), grid_cell(g, i, y1, k), c, s, a, xa, xaf, f);
        if (g.per[2] && (k == z0 || k == z1)) grid_all_in_cells(A, grid_cell(g, i, j, z0), grid_cell(g, i, j, z1), c, s, a, xa, xaf, f);
        if (g.per[0] && g.per[1] && ((i == x0 && j == y0) || (i == x1 && j == y1)))
            grid_all_in_cells(A, grid_cell(g, x0, y0, k), grid_cell(g, x1, y1, k), c, s, a, xa, xaf, f);
        if (g.per[0] && g.per[2] && ((i == x0 && k == z0) || (i == x1 && k == z1)))
            grid_all_in_cells(A, grid_cell(g, x0, j, z0), grid_cell(g, x1, j, z1), c, s, a, xa, xaf, f);
        if (g.per[1] && g.per[2] && ((j == y0 && k == z0) || (j == y1 && k == z1)))
            grid_all_in_cells(A, grid_cell(g, i, y0, z0), grid_cell(g, i, y1, z1), c, s, a, xa, xaf, f);
        if (g.per[0] && g.per[1] && g.per[2] && ((i == x0 && j == y0 && k == z0) || (i == x1 && j == y1 && k == z1)))
            grid_all_in_cells(A, grid_cell(g, x0, y0, z0), grid_cell(g, x1, y1, z1), c, s, a, xa, xaf, f);
        if (wr > 0) {
            // PipeBoundary::does_intersect(cell rect, cutoff) (Boundary.h:227-243), the rect of
            // Grid::repartition (Grid.hh:46-58)
            const double ry0 = add(g.b0[1], mul((double)(j - 1), g.cs[1])), ry1 = add(ry0, g.cs[1]);
            const double rz0 = add(g.b0[2], mul((double)(k - 1), g.cs[2])), rz1 = add(rz0, g.cs[2]);
            const double cy = sub(wy0, wy0 >= ry1 ? ry1 : (wy0 <= ry0 ? ry0 : wy0));
            const double cz = sub(wz0, wz0 >= rz1 ? rz1 : (wz0 <= rz0 ? rz0 : wz0));
            bool hit = false;
            if (add(mul(cy, cy), mul(cz, cz)) <= mul(wr, wr)) {
                const double rm = sub(wr, A.pot.r0), rm2 = mul(rm, rm);
                auto inside = [&](double y, double z) {
                    const double dy = sub(y, wy0), dz = sub(z, wz0);
                    return add(mul(dy, dy), mul(dz, dz)) < rm2;
                };
                hit = !(inside(ry0, rz0) && inside(ry0, rz1) && inside(ry1, rz0) && inside(ry1, rz1));
            }
            if (hit) {
                const double dy = sub(xa[1], wy0), dz = sub(xa[2], wz0);
                const double rr = __dsqrt_rn(add(mul(dy, dy), mul(dz, dz)));
                const double dist = sub(wr, rr);
                if (dist <= A.pot.r0) {
                    const double phi = grid_potential(A.pot, dist);
                    f[0] = sub(f[0], mul(phi, dvd(0.0, rr)));
                    f[1] = sub(f[1], mul(phi, dvd(dy, rr)));
                    f[2] = sub(f[2], mul(phi, dvd(dz, rr)));
                }
            }
        }
    }
    for (int d = 0; d < 3; ++d) fo[d] = f[d];
}

// ---------------------------------------------------------------- rigid growth
// Quaternion::to_rot_matrix (fsi/Quaternion.h:148-159)
__device__ void quat_matrix(const double* q, double* R) {
    R[0] = sub(1.0, mul(2.0, add(mul(q[2], q[2]), mul(q[3], q[3]))));
    R[1] = mul(2.0, sub(mul(q[1], q[2]), mul(q[0], q[3])));
    R[2] = mul(2.0, add(mul(q[0], q[2]), mul(q[1], q[3])));
    R[3] = mul(2.0, add(mul(q[1], q[2]), mul(q[0], q[3])));
    R[4] = sub(1.0, mul(2.0, add(mul(q[1], q[1]), mul(q[3], q[3]))));
    R[5] = mul(2.0, sub(mul(q[2], q[3]), mul(q[0], q[1])));
    R[6] = mul(2.0, sub(mul(q[1], q[3]), mul(q[0], q[2])));
    R[7] = mul(2.0, add(mul(q[0], q[1]), mul(q[2], q[3])));
    R[8] = sub(1.0, mul(2.0, add(mul(q[1], q[1]), mul(q[2], q[2]))));
}

__device__ __forceinline__ void mat_vec(const double* R, const double* w, double* r) {
    for (int d = 0; d < 3; ++d) r[d] = add(add(mul(R[3 * d], w[0]), mul(R[3 * d + 1], w[1])), mul(R[3 * d + 2], w[2]));
}

// RigidParticle3D::update (RigidParticle.hh:27-36): vertex i at com + R (scale v_i), plus shift
__device__ void rigid_vertices(const GrowthView& G, int p, const double* com, const double* R, double scale,
                               const double* shift) {
    const int s = G.shape[p];
    const double* v = G.verts + 3LL * G.shape_v0[s];
    double* x = G.pos + 3LL * G.part_v0[p];
    const int nv = G.shape_nv[s];
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        const double w[3] = {mul(scale, v[3 * i]), mul(scale, v[3 * i + 1]), mul(scale, v[3 * i + 2])};
        double r[3];
        mat_vec(R, w, r);
        for (int d = 0; d < 3; ++d) {
            const double y = add(com[d], r[d]);
            x[3 * i + d] = shift ? add(y, shift[d]) : y;
        }
    }
}

__global__ void __launch_bounds__(256) k_rigid_nodes(GrowthView G, double scale) {
    const int p = blockIdx.x;
    double R[9];
    quat_matrix(G.quat + 4LL * p, R);
    rigid_vertices(G, p, G.com + 3LL * p, R, scale, nullptr);
}

// The rescale of create_particles.h:132-147 at iterations it = 0, every, 2 every, ...: the
// iteration counter and the table of scales are in device memory, so a captured sequence of
// iterations replays unchanged.
__global__ void __launch_bounds__(256) k_rigid_rescale(GrowthView G) {
    const long long it = *G.it;
    if (it % G.every != 0) return;
    const double scale = G.scales[it / G.every];
    if (blockIdx.x == 0 && threadIdx.x == 0) *G.scale_now = scale;
    const int p = blockIdx.x;
    double R[9];
    quat_matrix(G.quat + 4LL * p, R);
    rigid_vertices(G, p, G.com + 3LL * p, R, scale, nullptr);
}

// RigidParticle3D::move_vertices (RigidParticle.hh:55-101) and the periodic remap of the
// centre of mass (ParticleBase.hh:111-136).
__global__ void __launch_bounds__(128) k_rigid_move(GrowthView G) {
    const int p = blockIdx.x;
    const double scale = *G.scale_now;
    __shared__ double sh[3 + 9 + 3];  // com before the remap, R, shift
    __shared__ double sums[6];        // force, torque
    const int s = G.shape[p];
    const int nv = G.shape_nv[s];
    const double* x = G.pos + 3LL * G.part_v0[p];
    const double* fr = G.force + 3LL * G.part_v0[p];
    double* tq = G.torque + 3LL * G.part_v0[p];
    // the torque terms (x_i - com) x f_i of all vertices at once; only their sums are ordered
    {
        const double* c = G.com + 3LL * p;
        for (int i = threadIdx.x; i < nv; i += blockDim.x) {
            const double f[3] = {fr[3 * i], fr[3 * i + 1], fr[3 * i + 2]};
            const double r[3] = {sub(x[3 * i], c[0]), sub(x[3 * i + 1], c[1]), sub(x[3 * i + 2], c[2])};
            tq[3 * i] = sub(mul(r[1], f[2]), mul(r[2], f[1]));
            tq[3 * i + 1] = sub(mul(r[2], f[0]), mul(r[0], f[2]));
            tq[3 * i + 2] = sub(mul(r[0], f[1]), mul(r[1], f[0]));
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {  // six running sums in vertex order, one per lane
        const double* src = threadIdx.x < 3 ? fr + threadIdx.x : tq + (threadIdx.x - 3);
        double acc = 0.0;
        for (int i = 0; i < nv; ++i) acc = add(acc, src[3 * i]);
        sums[threadIdx.x] = acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double* c = G.com + 3LL * p;
        double* q = G.quat + 4LL * p;
        double* v = G.vel + 3LL * p;
        double* w = G.omega + 3LL * p;
        const double F[3] = {sums[0], sums[1], sums[2]}, T[3] = {sums[3], sums[4], sums[5]};
        double R[9];
        quat_matrix(q, R);
        // apply_inv_rotation is R^T, apply_rotation R (Quaternion.h:102-146)
        auto rot_inv = [&](const double* a, double* r) {
            for (int d = 0; d < 3; ++d) r[d] = add(add(mul(R[d], a[0]), mul(R[3 + d], a[1])), mul(R[6 + d], a[2]));
        };
        double wb[3], tb[3], Ib[9];
        rot_inv(w, wb);
        // density * std::pow(scale, 5): the reference's C++98 build multiplies x^2 x^3
        const double s2 = mul(scale, scale), s3 = mul(scale, s2);
        const double fac = mul(G.density, mul(s2, s3));
        for (int k = 0; k < 9; ++k) Ib[k] = mul(fac, G.inertia[9 * s + k]);
        const double mass = mul(mul(mul(mul(scale, scale), scale), G.volume[s]), G.density);
        double Iw[3];
        mat_vec(Ib, wb, Iw);
        const double cw[3] = {sub(mul(wb[1], Iw[2]), mul(wb[2], Iw[1])), sub(mul(wb[2], Iw[0]), mul(wb[0], Iw[2])),
                              sub(mul(wb[0], Iw[1]), mul(wb[1], Iw[0]))};
        rot_inv(T, tb);
        const double rhs[3] = {sub(tb[0], cw[0]), sub(tb[1], cw[1]), sub(tb[2], cw[2])};
        // Matrix<T, 3>::solve (fsi/Matrix3.h:129-144)
        const double* m = Ib;
        // a - b - c + d + e - f, left to right
        const double detv = sub(add(add(sub(sub(mul(mul(m[0], m[4]), m[8]), mul(mul(m[0], m[5]), m[7])),
                                             mul(mul(m[1], m[3]), m[8])),
                                         mul(mul(m[1], m[5]), m[6])),
                                     mul(mul(m[2], m[3]), m[7])),
                                mul(mul(m[2], m[4]), m[6]));
        double sol[3];
        sol[0] = dvd(add(add(mul(rhs[2], sub(mul(m[1], m[5]), mul(m[2], m[4]))), mul(rhs[1], sub(mul(m[2], m[7]), mul(m[1], m[8])))),
                         mul(rhs[0], sub(mul(m[4], m[8]), mul(m[5], m[7])))),
                     detv);
        sol[1] = dvd(add(add(mul(rhs[2], sub(mul(m[2], m[3]), mul(m[0], m[5]))), mul(rhs[1], sub(mul(m[0], m[8]), mul(m[2], m[6])))),
                         mul(rhs[0], sub(mul(m[5], m[6]), mul(m[3], m[8])))),
                     detv);
        sol[2] = dvd(add(add(mul(rhs[2], sub(mul(m[0], m[4]), mul(m[1], m[3]))), mul(rhs[1], sub(mul(m[1], m[6]), mul(m[0], m[7])))),
                         mul(rhs[0], sub(mul(m[3], m[7]), mul(m[4], m[6])))),
                     detv);
        double rw[3];
        mat_vec(R, sol, rw);
        double vdot[3];
        for (int d = 0; d < 3; ++d) vdot[d] = sub(dvd(F[d], mass), mul(G.damping, v[d]));
        for (int d = 0; d < 3; ++d) {
            v[d] = add(v[d], vdot[d]);
            w[d] = add(w[d], sub(rw[d], mul(G.damping, w[d])));
        }
        for (int d = 0; d < 3; ++d) c[d] = add(c[d], v[d]);
        // unit-norm exponential map (RigidParticle.hh:90-94)
        const double wn = __dsqrt_rn(add(add(mul(w[0], w[0]), mul(w[1], w[1])), mul(w[2], w[2])));
        if (wn >= 10.0 * DBL_EPSILON) {
            const double ax[3] = {dvd(w[0], wn), dvd(w[1], wn), dvd(w[2], wn)};
            double sn, cs;
            sincos(dvd(wn, 2.0), &sn, &cs);
            const double r[4] = {cs, mul(sn, ax[0]), mul(sn, ax[1]), mul(sn, ax[2])};
            const double qn[4] = {
                sub(mul(r[0], q[0]), add(add(mul(r[1], q[1]), mul(r[2], q[2])), mul(r[3], q[3]))),
                sub(add(add(mul(r[0], q[1]), mul(q[0], r[1])), mul(r[2], q[3])), mul(r[3], q[2])),
                sub(add(add(mul(r[0], q[2]), mul(q[0], r[2])), mul(r[3], q[1])), mul(r[1], q[3])),
                sub(add(add(mul(r[0], q[3]), mul(q[0], r[3])), mul(r[1], q[2])), mul(r[2], q[1]))};
            for (int k = 0; k < 4; ++k) q[k] = qn[k];
        }
        quat_matrix(q, R);
        double np_[3] = {c[0], c[1], c[2]};
        for (int d = 0; d < 3; ++d)
            if (G.per[d]) np_[d] = sub(np_[d], mul(G.L[d], floor(mul(sub(np_[d], G.x0[d]), G.Linv[d]))));
        for (int d = 0; d < 3; ++d) {
            sh[d] = c[d];
            sh[12 + d] = sub(np_[d], c[d]);
            c[d] = np_[d];
        }
        for (int k = 0; k < 9; ++k) sh[3 + k] = R[k];
    }
    __syncthreads();
    rigid_vertices(G, p, sh, sh + 3, scale, sh + 12);
    if (p == 0 && threadIdx.x == 0) *G.it += 1;  // no other block reads the counter
}

}  // namespace

int64_t ref_grid_cells(const int64_t* box) {
    int64_t n = 1;
    for (int a = 0; a < 3; ++a) {
        const double b0 = (double)box[2 * a] - 0.5, b1 = (double)box[2 * a + 1] + 0.5 - DBL_EPSILON;
        n *= (int64_t)std::floor((b1 - b0) / 1.0) + 2;
    }
    return n;
}

RefGrid ref_grid(const int64_t* box, const int* periodic, double cut, int nvert) {
    RefGrid g{};
    g.ncell = 1;
    for (int a = 0; a < 3; ++a) {
        const int64_t lo = box[2 * a], hi = box[2 * a + 1];
        g.b0[a] = (double)lo - 0.5;
        const double b1 = (double)hi + 0.5 - DBL_EPSILON;
        const double nb = std::floor((b1 - g.b0[a]) / 1.0);
        g.cs[a] = (b1 - g.b0[a]) / nb;
        g.nc[a] = (int)nb + 2;
        g.g0[a] = g.b0[a] - g.cs[a];
        g.lo[a] = g.b0[a] - cut;
        g.hi[a] = b1 + cut;
        g.per[a] = periodic[a] ? 1 : 0;
        g.L[a] = (double)(hi - lo + 1);
        g.Linv[a] = 1. / g.L[a];
        g.ncell *= g.nc[a];
    }
    g.nvert = nvert;
    return g;
}

size_t ref_grid_temp_bytes(int nvert, int bits) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs((void*)nullptr, bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, nvert, 0, bits);
    return bytes;
}

int ref_grid_bits(int64_t ncell) {
    int bits = 1;
    while (((int64_t)1 << bits) <= ncell) ++bits;  // the sentinel ncell needs a key too
    return bits;
}

void launch_ref_grid_forces(const RefGrid& g, const RefGridBuffers& B, const PotentialDev& pot, const double* pos,
                            const int* owner, double* force, bool zero, const double* wall, cudaStream_t s) {
    const int n = g.nvert;
    if (n <= 0) return;
    const unsigned b = (unsigned)((n + 127) / 128);
    k_grid_clear<<<b, 128, 0, s>>>(n, B.keys[1], B.start, B.end);
    k_grid_keys<<<b, 128, 0, s>>>(g, n, pos, B.keys[0], B.ids[0], B.posf);
    size_t tb = B.temp_bytes;
    cub::DeviceRadixSort::SortPairs(B.temp, tb, B.keys[0], B.keys[1], B.ids[0], B.ids[1], n, 0, B.bits, s);
    k_grid_bounds<<<b, 128, 0, s>>>(n, B.keys[1], B.start, B.end);
    GridArgs A{};
    A.g = g;
    A.pot = pot;
    A.c2 = pot.r0 * pot.r0;
    A.pos = pos;
    A.posf = B.posf;
    A.owner = owner;
    A.keys = B.keys[1];
    A.ids = B.ids[1];
    A.start = B.start;
    A.end = B.end;
    // margin of the FP32 pre-test: the rounding of coordinates up to X (the box and its envelope)
    // to FP32, twice, with a factor 4 of slack
    double X = 0.0;
    bool small_period = false;
    for (int d = 0; d < 3; ++d) {
        X = std::max(X, std::max(std::fabs(g.b0[d]), std::fabs(g.b0[d] + g.L[d])) + 4.0);
        A.Lf[d] = (float)g.L[d];
        A.Linvf[d] = (float)g.Linv[d];
        small_period = small_period || (g.per[d] && g.L[d] < 2.0 * pot.r0 + 4.0);
    }
    const double margin = 8.0 * X * std::ldexp(1.0, -24) + 1e-4;
    A.pre_c2 = small_period ? 0.0f : (float)((pot.r0 + margin) * (pot.r0 + margin) * (1.0 + 1e-6));
    const double wy0 = wall ? wall[0] : 0.0, wz0 = wall ? wall[1] : 0.0, wr = wall ? wall[2] : -1.0;
    // FP64-bound threads: with few vertices, one warp per CTA spreads them over more SMs
    const int tpb = n < 152 * 128 ? 32 : 128;
    const unsigned bf = (unsigned)((n + tpb - 1) / tpb);
    if (zero) k_grid_forces<true><<<bf, tpb, 0, s>>>(A, wy0, wz0, wr, force);
    else k_grid_forces<false><<<bf, tpb, 0, s>>>(A, wy0, wz0, wr, force);
}

void launch_rigid_nodes(const GrowthView& G, double scale, cudaStream_t s) {
    if (G.np > 0) k_rigid_nodes<<<G.np, 256, 0, s>>>(G, scale);
}

void launch_rigid_rescale(const GrowthView& G, cudaStream_t s) {
    if (G.np > 0) k_rigid_rescale<<<G.np, 256, 0, s>>>(G);
}

void launch_rigid_move(const GrowthView& G, cudaStream_t s) {
    if (G.np > 0) k_rigid_move<<<G.np, 128, 0, s>>>(G);
}

}  // namespace bib
