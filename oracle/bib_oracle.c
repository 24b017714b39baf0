/*
 * bib_oracle.c -- CPU restatement of the reference's hot IB-LBM step (FP64).
 *
 * TEST INFRASTRUCTURE ONLY (see bib_oracle.h).  Compiled with -ffp-contract=off so
 * that every product / sum is rounded as in the reference build.
 *
 * Reference paths below are relative to the niclasberg/biblbm checkout.
 */
#include "bib_oracle.h"

#include <float.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdlib.h>
#include <string.h>

#define Q 19

/* D3Q19 velocity set and weights in the reference order,
 * src/latticeBoltzmann/nearestNeighborLattices3D.hh:165-197 (c[i] = -c[i+9]). */
static const int CX[Q] = {0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0};
static const int CY[Q] = {0, 0, -1, 0, -1, 1, 0, 0, -1, -1, 0, 1, 0, 1, -1, 0, 0, 1, 1};
static const int CZ[Q] = {0, 0, 0, -1, 0, 0, -1, 1, -1, 1, 0, 0, 1, 0, 0, 1, -1, 1, -1};
static double TW[Q];
static int tw_ready = 0;
static void init_weights(void) {
    if (tw_ready) return;
    TW[0] = (double)1 / (double)3;
    for (int i = 1; i < Q; ++i) {
        int n2 = CX[i] * CX[i] + CY[i] * CY[i] + CZ[i] * CZ[i];
        TW[i] = n2 == 1 ? (double)1 / (double)18 : (double)1 / (double)36;
    }
    tw_ready = 1;
}
static int opp(int i) { return i == 0 ? 0 : (i < 10 ? i + 9 : i - 9); }

static inline int64_t cell_index(const orc_lattice* L, int64_t x, int64_t y, int64_t z) {
    return x + L->nx * (y + L->ny * z);
}

/* ------------------------------------------------------------------ moments */
/* momentTemplatesImpl<T, D3Q19DescriptorBase>::get_rhoBar, momentTemplates3D.h:375-382 */
static double get_rhoBar(const double* f) {
    double r = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11] + f[12] +
               f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
    return r;
}

/* partial_rho + get_rhoBar_j, momentTemplates3D.h:350-372 and 411-423 */
static void get_rhoBar_j(const double* f, double* rhoBar, double* j) {
    double sxm = f[1] + f[4] + f[5] + f[6] + f[7];
    double sxp = f[10] + f[13] + f[14] + f[15] + f[16];
    double sym = f[2] + f[4] + f[8] + f[9] + f[14];
    double syp = f[5] + f[11] + f[13] + f[17] + f[18];
    double szm = f[3] + f[6] + f[8] + f[16] + f[18];
    double szp = f[7] + f[9] + f[12] + f[15] + f[17];
    double sx0 = f[0] + f[2] + f[3] + f[8] + f[9] + f[11] + f[12] + f[17] + f[18];
    *rhoBar = sxm + sx0 + sxp;
    j[0] = sxp - sxm;
    j[1] = syp - sym;
    j[2] = szp - szm;
}

/* ExternalForceDynamics::computeVelocity, basicDynamics/externalForceDynamics.hh:59-74:
 * u = j/rho + F/2 with rho from the partial sums. */
static void velocity_with_force(const double* f, const double* F, double* u) {
    double rb, j[3];
    get_rhoBar_j(f, &rb, j);
    double invRho = (double)1 / (rb + (double)1);
    for (int d = 0; d < 3; ++d) u[d] = j[d] * invRho + F[d] / (double)2;
}

/* ------------------------------------------------------------------ collision */
/* dynamicsTemplatesImpl<T, D3Q19DescriptorBase>::bgk_ma2_collision_base,
 * latticeBoltzmann/dynamicsTemplates3D.h:770-838 */
static void bgk_ma2_collision_base(double* f, double rhoBar, const double* j, double omega, double invRho) {
    const double one_m_omega = (double)1 - omega;
    const double t0_omega = TW[0] * omega, t1_omega = TW[1] * omega, t4_omega = TW[4] * omega;
    const double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    const double kx = (double)3 * j[0], ky = (double)3 * j[1], kz = (double)3 * j[2];
    const double kxSqr_ = invRho / (double)2 * kx * kx;
    const double kySqr_ = invRho / (double)2 * ky * ky;
    const double kzSqr_ = invRho / (double)2 * kz * kz;
    const double kxky_ = invRho * kx * ky;
    const double kxkz_ = invRho * kx * kz;
    const double kykz_ = invRho * ky * kz;
    const double C1 = rhoBar + invRho * (double)3 * jSqr;
    double C2, C3;
    C3 = -kxSqr_ - kySqr_ - kzSqr_;
    f[0] *= one_m_omega; f[0] += t0_omega * (C1 + C3);
#define PAIR(a, b, tw) f[a] *= one_m_omega; f[a] += tw * (C1 + C2 + C3); f[b] *= one_m_omega; f[b] += tw * (C1 - C2 + C3);
    C2 = -kx; C3 = -kySqr_ - kzSqr_; PAIR(1, 10, t1_omega)
    C2 = -ky; C3 = -kxSqr_ - kzSqr_; PAIR(2, 11, t1_omega)
    C2 = -kz; C3 = -kxSqr_ - kySqr_; PAIR(3, 12, t1_omega)
    C2 = -kx - ky; C3 = kxky_ - kzSqr_; PAIR(4, 13, t4_omega)
    C2 = -kx + ky; C3 = -kxky_ - kzSqr_; PAIR(5, 14, t4_omega)
    C2 = -kx - kz; C3 = kxkz_ - kySqr_; PAIR(6, 15, t4_omega)
    C2 = -kx + kz; C3 = -kxkz_ - kySqr_; PAIR(7, 16, t4_omega)
    C2 = -ky - kz; C3 = kykz_ - kxSqr_; PAIR(8, 17, t4_omega)
    C2 = -ky + kz; C3 = -kykz_ - kxSqr_; PAIR(9, 18, t4_omega)
#undef PAIR
}

/* bgk_ma2_equilibrium, dynamicsTemplates3D.h:675-678 */
static double bgk_ma2_equilibrium(int i, double rhoBar, double invRho, const double* j, double jSqr) {
    double c_j = CX[i] * j[0] + CY[i] * j[1] + CZ[i] * j[2];
    return TW[i] * (rhoBar + 3. * c_j + invRho * (4.5 * c_j * c_j - 1.5 * jSqr));
}

/* vofTemplatesImpl<T, ForcedPhaseD3Q19Descriptor>::addGuoForce, fsi/VariableViscosityDynamics.hh:47-129 */
static void add_guo_force(double* f, const double* force, const double* u, double omega, double amplitude) {
    const double mu = amplitude * ((double)1 - omega / (double)2);
    const double oneOver6 = (double)1 / (double)6;
    const double oneOver12 = (double)1 / (double)12;
    f[0] += -mu * (force[0] * u[0] + force[1] * u[1] + force[2] * u[2]);
    f[1] += oneOver6 * mu * (force[0] * (-(double)1 + 2 * u[0]) - force[1] * u[1] - force[2] * u[2]);
    f[2] += -oneOver6 * mu * (force[0] * u[0] + force[1] * ((double)1 - 2 * u[1]) + force[2] * u[2]);
    f[3] += -oneOver6 * mu * (force[0] * u[0] + force[1] * u[1] + force[2] * ((double)1 - 2 * u[2]));
    f[4] += oneOver12 * mu * (force[0] * (-(double)1 + 2 * u[0] + 3 * u[1]) + force[1] * (-(double)1 + 2 * u[1] + 3 * u[0]) - force[2] * u[2]);
    f[5] += oneOver12 * mu * (force[0] * (-(double)1 + 2 * u[0] - 3 * u[1]) + force[1] * ((double)1 + 2 * u[1] - 3 * u[0]) - force[2] * u[2]);
    f[6] += oneOver12 * mu * (force[0] * (-(double)1 + 2 * u[0] + 3 * u[2]) - force[1] * u[1] + force[2] * (-(double)1 + 2 * u[2] + 3 * u[0]));
    f[7] += oneOver12 * mu * (force[0] * (-(double)1 + 2 * u[0] - 3 * u[2]) - force[1] * u[1] + force[2] * ((double)1 + 2 * u[2] - 3 * u[0]));
    f[8] += -oneOver12 * mu * (force[0] * u[0] + force[1] * ((double)1 - 2 * u[1] - 3 * u[2]) + force[2] * ((double)1 - 2 * u[2] - 3 * u[1]));
    f[9] += -oneOver12 * mu * (force[0] * u[0] + force[1] * ((double)1 - 2 * u[1] + 3 * u[2]) + force[2] * (-(double)1 - 2 * u[2] + 3 * u[1]));
    f[10] += oneOver6 * mu * (force[0] * ((double)1 + 2 * u[0]) - force[1] * u[1] - force[2] * u[2]);
    f[11] += -oneOver6 * mu * (force[0] * u[0] + force[1] * (-(double)1 - 2 * u[1]) + force[2] * u[2]);
    f[12] += -oneOver6 * mu * (force[0] * u[0] + force[1] * u[1] + force[2] * (-(double)1 - 2 * u[2]));
    f[13] += oneOver12 * mu * (force[0] * ((double)1 + 2 * u[0] + 3 * u[1]) + force[1] * ((double)1 + 2 * u[1] + 3 * u[0]) - force[2] * u[2]);
    f[14] += oneOver12 * mu * (force[0] * ((double)1 + 2 * u[0] - 3 * u[1]) + force[1] * (-(double)1 + 2 * u[1] - 3 * u[0]) - force[2] * u[2]);
    f[15] += oneOver12 * mu * (force[0] * ((double)1 + 2 * u[0] + 3 * u[2]) - force[1] * u[1] + force[2] * ((double)1 + 2 * u[2] + 3 * u[0]));
    f[16] += oneOver12 * mu * (force[0] * ((double)1 + 2 * u[0] - 3 * u[2]) - force[1] * u[1] + force[2] * (-(double)1 + 2 * u[2] - 3 * u[0]));
    f[17] += -oneOver12 * mu * (force[0] * u[0] + force[1] * (-(double)1 - 2 * u[1] - 3 * u[2]) + force[2] * (-(double)1 - 2 * u[2] - 3 * u[1]));
    f[18] += -oneOver12 * mu * (force[0] * u[0] + force[1] * (-(double)1 - 2 * u[1] + 3 * u[2]) + force[2] * ((double)1 - 2 * u[2] + 3 * u[1]));
}

/* Two-relaxation-time collision (no reference counterpart: the reference has BGK only).
 * Ginzburg's symmetric / antisymmetric split with the magic parameter
 * Lambda = (1/w+ - 1/2)(1/w- - 1/2); the equilibrium is the reference's
 * bgk_ma2_equilibrium so both operators share one storage convention. */
static void trt_collision(double* f, double omega, double magic) {
    double rb, j[3];
    get_rhoBar_j(f, &rb, j);
    const double invRho = 1.0 / (rb + 1.0);
    const double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    const double omega_m = 1.0 / (magic / (1.0 / omega - 0.5) + 0.5);
    double eq[Q];
    for (int i = 0; i < Q; ++i) eq[i] = bgk_ma2_equilibrium(i, rb, invRho, j, jSqr);
    f[0] = f[0] - omega * (f[0] - eq[0]);
    for (int i = 1; i < 10; ++i) {
        const int o = i + 9;
        const double fp = 0.5 * (f[i] + f[o]), fm = 0.5 * (f[i] - f[o]);
        const double ep = 0.5 * (eq[i] + eq[o]), em = 0.5 * (eq[i] - eq[o]);
        const double dp = omega * (fp - ep), dm = omega_m * (fm - em);
        f[i] = f[i] - dp - dm;
        f[o] = f[o] - dp + dm;
    }
}

void orc_collide_cell(const orc_lattice* L, double* f, const double* F, double phase) {
    init_weights();
    if (L->collision == ORC_COLLISION_BGK_GUO_VOF) {
        /* GuoExternalForceVOFDynamics::collide, fsi/VariableViscosityDynamics.hh:151-172 */
        const double rhoBar = get_rhoBar(f);
        double u[3], j[3];
        velocity_with_force(f, F, u);
        const double rho = rhoBar + (double)1;
        for (int d = 0; d < 3; ++d) j[d] = rho * u[d];
        /* computeOmega, VariableViscosityDynamics.hh:131-141 */
        const double c = phase;
        const double omega = L->omega * L->omega_inner / (c * L->omega + ((double)1. - c) * L->omega_inner);
        bgk_ma2_collision_base(f, rhoBar, j, omega, (double)1 / (rhoBar + (double)1));
        add_guo_force(f, F, u, omega, (double)1);
    } else if (L->collision == ORC_COLLISION_BGK) {
        /* BGKdynamics::collide, basicDynamics/isoThermalDynamics.hh:329-340 */
        double rb, j[3];
        get_rhoBar_j(f, &rb, j);
        bgk_ma2_collision_base(f, rb, j, L->omega, (double)1 / (rb + (double)1));
    } else {
        trt_collision(f, L->omega, L->trt_magic);
    }
}

/* ------------------------------------------------------------------ voxelization */
/* RayTracer::tri_ray_intersect (fsi/RayTracer.hh:80-108) for the ray from (px, py, 0) along +z,
 * Moller-Trumbore with Palabos' crossProduct / dot (geometricOperationTemplates.h:460-480). */
static int tri_ray_z(const double* v0, const double* v1, const double* v2, double px, double py, double* dist) {
    const double e1[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    const double e2[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
    const double dir[3] = {0.0, 0.0, 1.0};
    const double q[3] = {dir[1] * e2[2] - dir[2] * e2[1], dir[2] * e2[0] - dir[0] * e2[2], dir[0] * e2[1] - dir[1] * e2[0]};
    double a = 0.0;
    for (int d = 0; d < 3; ++d) a += e1[d] * q[d];
    if (fabs(a) < DBL_EPSILON) return 0;
    const double f = 1 / a;
    const double sv[3] = {px - v0[0], py - v0[1], 0.0 - v0[2]};
    double sq = 0.0;
    for (int d = 0; d < 3; ++d) sq += sv[d] * q[d];
    const double u = f * sq;
    if (u < 0.0) return 0;
    const double r[3] = {sv[1] * e1[2] - sv[2] * e1[1], sv[2] * e1[0] - sv[0] * e1[2], sv[0] * e1[1] - sv[1] * e1[0]};
    double dr = 0.0;
    for (int d = 0; d < 3; ++d) dr += dir[d] * r[d];
    const double v = f * dr;
    if (v < 0.0 || u + v > 1.0) return 0;
    double er = 0.0;
    for (int d = 0; d < 3; ++d) er += e2[d] * r[d];
    *dist = f * er;
    return 1;
}

static int cmp_double(const void* a, const void* b) {
    const double x = *(const double*)a, y = *(const double*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* ImmersedBoundaryDynamics3D::voxelize + apply_voxelization
 * (fsi/ImmersedBoundaryDynamics_voxelization.hh:17-30, 121-161): every triangle casts z-rays
 * through the integer (x, y) points of its xy bounding box (RayTracer::find_intersections_z,
 * RayTracer.hh:18-40); the intersection heights go into the ZBuffer column of (x, y) (periodic
 * index and height wrap, ZBuffer.h put / Periodicity.h:83-93, heights in [-1/2, nz - 1/2)); each
 * column is sorted and filled from below by parity, [ceil(z_prev), floor(z)] getting the current
 * inside flag; above the last intersection the fill only happens when ceil(z_last) < nz - 1. */
void orc_voxelize(const orc_lattice* L, int64_t nvt, const double* pos, int64_t ntt, const int64_t* tri, double* phase) {
    (void)nvt;
    const int64_t nx = L->nx, ny = L->ny, nz = L->nz, ncol = nx * ny;
    int64_t* count = (int64_t*)calloc((size_t)ncol + 1, sizeof(int64_t));
    /* two passes over the triangles: count, then fill */
    double* zs = NULL;
    int64_t* fillp = NULL;
    for (int pass = 0; pass < 2; ++pass) {
        for (int64_t t = 0; t < ntt; ++t) {
            const double* v0 = pos + 3 * tri[3 * t];
            const double* v1 = pos + 3 * tri[3 * t + 1];
            const double* v2 = pos + 3 * tri[3 * t + 2];
            const int64_t i0 = (int64_t)ceil(fmin(v0[0], fmin(v1[0], v2[0])));
            const int64_t i1 = (int64_t)floor(fmax(v0[0], fmax(v1[0], v2[0])));
            const int64_t j0 = (int64_t)ceil(fmin(v0[1], fmin(v1[1], v2[1])));
            const int64_t j1 = (int64_t)floor(fmax(v0[1], fmax(v1[1], v2[1])));
            for (int64_t i = i0; i <= i1; ++i)
                for (int64_t j = j0; j <= j1; ++j) {
                    double dist;
                    if (!tri_ray_z(v0, v1, v2, (double)i, (double)j, &dist)) continue;
                    int64_t cx = i, cy = j;
                    if (L->periodic[0]) cx = ((cx % nx) + nx) % nx;
                    else if (cx < 0 || cx >= nx) continue;
                    if (L->periodic[1]) cy = ((cy % ny) + ny) % ny;
                    else if (cy < 0 || cy >= ny) continue;
                    /* Arithmetic1D::remap_pos with the periodic interval [-1/2, nz - 1/2),
                     * Periodicity.h:83-87 (x0 = -0.5, as for the centre-of-mass remap) */
                    if (L->periodic[2]) dist = dist - (double)nz * floor((dist - (-0.5)) * (1.0 / (double)nz));
                    const int64_t c = cx * ny + cy;
                    if (pass == 0) count[c + 1]++;
                    else zs[fillp[c]++] = dist;
                }
        }
        if (pass == 0) {
            for (int64_t c = 0; c < ncol; ++c) count[c + 1] += count[c];
            zs = (double*)malloc(sizeof(double) * (size_t)(count[ncol] > 0 ? count[ncol] : 1));
            fillp = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncol);
            for (int64_t c = 0; c < ncol; ++c) fillp[c] = count[c];
        }
    }
    for (int64_t cx = 0; cx < nx; ++cx)
        for (int64_t cy = 0; cy < ny; ++cy) {
            const int64_t c = cx * ny + cy;
            double* col = zs + count[c];
            const int64_t m = count[c + 1] - count[c];
            qsort(col, (size_t)m, sizeof(double), cmp_double);
            int inside = 0;
            double z_last = -10000;
            for (int64_t e = 0; e <= m; ++e) {
                int64_t lo, hi;
                if (e < m) {
                    lo = (int64_t)ceil(z_last); if (lo < 0) lo = 0;
                    hi = (int64_t)floor(col[e]); if (hi > nz - 1) hi = nz - 1;
                } else {
                    if (!(ceil(z_last) < (double)(nz - 1))) break;
                    lo = (int64_t)ceil(z_last); if (lo < 0) lo = 0;
                    hi = nz - 1;
                }
                for (int64_t z = lo; z <= hi; ++z) phase[cell_index(L, cx, cy, z)] = inside ? 1.0 : 0.0;
                if (e < m) {
                    z_last = col[e];
                    inside = !inside;
                }
            }
        }
    free(count);
    free(zs);
    free(fillp);
}

/* ------------------------------------------------------------------ walls */
static int is_fd_wall(const orc_lattice* L, int64_t y, int64_t z) {
    if (!L->periodic[1] && L->wall_y == ORC_WALL_FD_VELOCITY && (y == 0 || y == L->ny - 1)) return 1;
    if (!L->periodic[2] && L->wall_z == ORC_WALL_FD_VELOCITY && (z == 0 || z == L->nz - 1)) return 1;
    return 0;
}

static const double* fd_wall_velocity(const orc_lattice* L, int64_t y, int64_t z) {
    if (!L->periodic[1] && L->wall_y == ORC_WALL_FD_VELOCITY) {
        if (y == 0) return L->wall_u[0];
        if (y == L->ny - 1) return L->wall_u[1];
    }
    return z == 0 ? L->wall_u[2] : L->wall_u[3];
}

/* fromPiToFneq (generic), latticeBoltzmann/offEquilibriumTemplates.h:91-115.
 * pi order: xx, xy, xz, yy, yz, zz. */
static double from_pi_to_fneq(int i, const double* pi) {
    const int c[3] = {CX[i], CY[i], CZ[i]};
    const double cs2 = (double)1 / (double)3, invCs2 = (double)3;
    double fNeq = 0.0;
    int iPi = 0;
    for (int a = 0; a < 3; ++a) {
        fNeq += pi[iPi] * (c[a] * c[a] - cs2);
        ++iPi;
        for (int b = a + 1; b < 3; ++b) {
            fNeq += pi[iPi] * (double)2 * c[a] * c[b];
            ++iPi;
        }
    }
    fNeq *= TW[i] * invCs2 * invCs2 / (double)2;
    return fNeq;
}

/* PlaneFdBoundaryFunctional3D::processCell for a y-normal plane,
 * boundaryCondition/finiteDifferenceBoundaryProcessor3D.hh:68-115, with the density of
 * VelocityDirichletBoundaryDynamics::computeRhoBar (boundaryDynamics.hh:631-663) and the
 * one-sided normal derivative of fd::DirectedGradients3D::o1_velocityDerivative
 * (finiteDifference/finiteDifference3D.h:67-82).  The wall velocity is uniform along the
 * plane, so the tangential central differences are exactly zero. */
static void fd_wall_cell(const orc_lattice* L, double* f, const double* F, int64_t x, int64_t y, int64_t z,
                         int orientation, const double* uw) {
    const int64_t n = L->nx * L->ny * L->nz;
    const int64_t k = cell_index(L, x, y, z);
    double fc[Q];
    for (int i = 0; i < Q; ++i) fc[i] = f[i * n + k];
    double Fc[3] = {F[k], F[n + k], F[2 * n + k]};
    /* density from the populations on the wall plane and those leaving through it */
    double rhoOnWall = 0.0, rhoNormal = 0.0;
    for (int i = 0; i < Q; ++i) {
        if (CY[i] == 0) rhoOnWall += fc[i];
    }
    for (int i = 0; i < Q; ++i) {
        if (CY[i] == orientation) rhoNormal += fc[i];
    }
    const double velNormal = (double)orientation * (uw[1] - 0.5 * Fc[1]);
    const double rhoBarW = ((double)2 * rhoNormal + rhoOnWall - (double)1 * velNormal) / ((double)1 + velNormal);
    const double rho = rhoBarW + (double)1;
    /* velocity one node into the fluid */
    const int64_t k1 = cell_index(L, x, y - orientation, z);
    double f1[Q], F1[3], u1[3];
    for (int i = 0; i < Q; ++i) f1[i] = f[i * n + k1];
    for (int d = 0; d < 3; ++d) F1[d] = F[d * n + k1];
    velocity_with_force(f1, F1, u1);
    double dy_u[3];
    for (int d = 0; d < 3; ++d) dy_u[d] = (double)(-orientation) * (u1[d] - uw[d]);
    const double dx_u[3] = {0.0, 0.0, 0.0}, dz_u[3] = {0.0, 0.0, 0.0};
    const double omega = L->omega;
    const double sToPi = -rho / (double)3 / omega;
    double pi[6];
    pi[0] = (double)2 * dx_u[0] * sToPi;
    pi[3] = (double)2 * dy_u[1] * sToPi;
    pi[5] = (double)2 * dz_u[2] * sToPi;
    pi[1] = (dx_u[1] + dy_u[0]) * sToPi;
    pi[2] = (dx_u[2] + dz_u[0]) * sToPi;
    pi[4] = (dy_u[2] + dz_u[1]) * sToPi;
    double j[3];
    for (int d = 0; d < 3; ++d) j[d] = rho * uw[d];
    const double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    const double rhoBar = rho - (double)1;
    const double invRho = (double)1 / (rhoBar + (double)1);
    for (int i = 0; i < Q; ++i) f[i * n + k] = bgk_ma2_equilibrium(i, rhoBar, invRho, j, jSqr) + from_pi_to_fneq(i, pi);
}

void orc_apply_fd_walls(const orc_lattice* L, double* f, const double* F) {
    init_weights();
    if (L->periodic[1] || L->wall_y != ORC_WALL_FD_VELOCITY) return;
    /* bottom plane (addVelocityBoundary1N) then top plane (1P), shear_flow_setup.h:86-87 */
    for (int side = 0; side < 2; ++side) {
        const int64_t y = side == 0 ? 0 : L->ny - 1;
        const int orientation = side == 0 ? -1 : 1;
        for (int64_t x = 0; x < L->nx; ++x)
            for (int64_t z = 0; z < L->nz; ++z) fd_wall_cell(L, f, F, x, y, z, orientation, L->wall_u[side]);
    }
}

/* ------------------------------------------------------------------ collide + stream */
static int64_t wrap(int64_t i, int64_t n) { return ((i % n) + n) % n; }

void orc_collide_stream(const orc_lattice* L, double* f, double* ftmp, const double* F, const double* phase) {
    init_weights();
    const int64_t nx = L->nx, ny = L->ny, nz = L->nz, n = nx * ny * nz;
    memcpy(ftmp, f, sizeof(double) * Q * n);
    /* cells are independent and every (population, destination) pair is written once:
     * the z slabs run in parallel without changing any result */
#pragma omp parallel for schedule(static) if (n > 262144)
    for (int64_t z = 0; z < nz; ++z)
        for (int64_t y = 0; y < ny; ++y)
            for (int64_t x = 0; x < nx; ++x) {
                const int64_t k = cell_index(L, x, y, z);
                double fc[Q], Fc[3];
                for (int i = 0; i < Q; ++i) fc[i] = f[i * n + k];
                for (int d = 0; d < 3; ++d) Fc[d] = F ? F[d * n + k] : 0.0;
                /* Reference quirk, reproduced on request: Palabos rebuilds the dynamics of
                 * the periodic envelope cells from their serialised parameters, and
                 * TwoParamDynamicsGenerator (core/dynamicsIdentifiers.h:133-140) reads the two
                 * omegas as two arguments of one constructor call, whose evaluation order C++
                 * leaves unspecified; g++ on x86-64 swaps them.  Populations that cross a
                 * periodic face are collided in those envelope copies, i.e. with omega and
                 * omega_inner exchanged.  Invisible when omega == omega_inner. */
                double fsw[Q];
                const int edge = (L->periodic[0] && (x == 0 || x == nx - 1)) || (L->periodic[1] && (y == 0 || y == ny - 1)) ||
                                 (L->periodic[2] && (z == 0 || z == nz - 1));
                const int ct = L->celltype ? L->celltype[k] : ORC_CELL_FLUID;
                if (ct == ORC_CELL_BOUNCE_BACK) {
                    /* BounceBack::collide swaps each population with its opposite,
                     * core/dynamics.hh:763-770 */
                    for (int i = 1; i <= Q / 2; ++i) {
                        const double t = fc[i];
                        fc[i] = fc[i + Q / 2];
                        fc[i + Q / 2] = t;
                    }
                    for (int i = 0; i < Q; ++i) fsw[i] = fc[i];
                } else if (ct == ORC_CELL_NO_DYNAMICS) {
                    /* NoDynamics::collide leaves the populations unchanged */
                    for (int i = 0; i < Q; ++i) fsw[i] = fc[i];
                } else {
                    if (L->envelope_swap && edge) {
                        orc_lattice Ls = *L;
                        Ls.omega = L->omega_inner;
                        Ls.omega_inner = L->omega;
                        for (int i = 0; i < Q; ++i) fsw[i] = fc[i];
                        orc_collide_cell(&Ls, fsw, Fc, phase ? phase[k] : 0.0);
                    }
                    orc_collide_cell(L, fc, Fc, phase ? phase[k] : 0.0);
                }
                for (int i = 0; i < Q; ++i) {
                    int64_t xd = x + CX[i], yd = y + CY[i], zd = z + CZ[i];
                    const int crosses = (L->periodic[0] && (xd < 0 || xd >= nx)) || (L->periodic[1] && (yd < 0 || yd >= ny)) ||
                                        (L->periodic[2] && (zd < 0 || zd >= nz));
                    int out = 0;
                    int bb_face = -1;
                    if (L->periodic[0]) xd = wrap(xd, nx); else if (xd < 0 || xd >= nx) out = 1;
                    if (L->periodic[1]) yd = wrap(yd, ny);
                    else if (yd < 0 || yd >= ny) { out = 1; bb_face = yd < 0 ? 0 : 1; }
                    if (L->periodic[2]) zd = wrap(zd, nz);
                    else if (zd < 0 || zd >= nz) { out = 1; if (bb_face < 0) bb_face = zd < 0 ? 2 : 3; }
                    if (!out) {
                        ftmp[i * n + cell_index(L, xd, yd, zd)] = (L->envelope_swap && crosses) ? fsw[i] : fc[i];
                        continue;
                    }
                    /* Leaving the domain.  FD velocity walls: the population is lost and the
                     * wall processor rebuilds the wall node.  Halfway bounce-back: it returns to
                     * its node reversed, with the moving-wall term -6 t_i rho_w (c_i . u_w),
                     * rho_w = 1 (Ladd).  Unknown walls behave like FD walls. */
                    const int wall = (bb_face <= 1) ? L->wall_y : L->wall_z;
                    if (wall == ORC_WALL_HALFWAY_BB && bb_face >= 0) {
                        const double* uw = L->wall_u[bb_face];
                        const double cu = CX[i] * uw[0] + CY[i] * uw[1] + CZ[i] * uw[2];
                        ftmp[opp(i) * n + k] = fc[i] - 6.0 * TW[i] * cu;
                    }
                }
            }
    memcpy(f, ftmp, sizeof(double) * Q * n);
    orc_apply_fd_walls(L, f, F);
    if (L->guo) orc_apply_guo(L, f);
}

void orc_compute_velocity(const orc_lattice* L, const double* f, const double* F, double* u) {
    init_weights();
    const int64_t nx = L->nx, ny = L->ny, nz = L->nz, n = nx * ny * nz;
#pragma omp parallel for schedule(static) if (n > 262144)
    for (int64_t z = 0; z < nz; ++z)
        for (int64_t y = 0; y < ny; ++y)
            for (int64_t x = 0; x < nx; ++x) {
                const int64_t k = cell_index(L, x, y, z);
                double uc[3];
                if (L->celltype && L->celltype[k] != ORC_CELL_FLUID) {
                    /* BounceBack / NoDynamics::computeVelocity yield 0, core/dynamics.hh:796-801 */
                    uc[0] = uc[1] = uc[2] = 0.0;
                } else if (is_fd_wall(L, y, z)) {
                    /* StoreVelocityDynamics::computeVelocity returns the imposed velocity,
                     * boundaryCondition/boundaryDynamics.hh:316-322 */
                    const double* uw = fd_wall_velocity(L, y, z);
                    for (int d = 0; d < 3; ++d) uc[d] = uw[d];
                } else {
                    double fc[Q], Fc[3];
                    for (int i = 0; i < Q; ++i) fc[i] = f[i * n + k];
                    for (int d = 0; d < 3; ++d) Fc[d] = F ? F[d * n + k] : 0.0;
                    velocity_with_force(fc, Fc, uc);
                }
                for (int d = 0; d < 3; ++d) u[d * n + k] = uc[d];
            }
}

/* iniCellAtEquilibrium, core/cell.hh:124-132 */
void orc_init_equilibrium(const orc_lattice* L, double* f, const double* rho, const double* u) {
    init_weights();
    const int64_t n = L->nx * L->ny * L->nz;
    for (int64_t k = 0; k < n; ++k) {
        const double r = rho ? rho[k] : 1.0;
        double j[3] = {u[k] * r, u[n + k] * r, u[2 * n + k] * r};
        const double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
        const double rhoBar = r - (double)1;
        const double invRho = (double)1 / (rhoBar + (double)1);
        for (int i = 0; i < Q; ++i) f[i * n + k] = bgk_ma2_equilibrium(i, rhoBar, invRho, j, jSqr);
    }
}

/* ------------------------------------------------------------------ small vector helpers
 * Palabos Array arithmetic: norm = sqrt(x0*x0 + x1*x1 + x2*x2), crossProduct and dot in
 * component order (core/array.h, latticeBoltzmann/geometricOperationTemplates.h). */
typedef struct { double v[3]; } v3;
static inline v3 mk(double a, double b, double c) { v3 r = {{a, b, c}}; return r; }
static inline v3 ld(const double* p) { return mk(p[0], p[1], p[2]); }
static inline v3 sub(v3 a, v3 b) { return mk(a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]); }
static inline v3 add(v3 a, v3 b) { return mk(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }
static inline v3 scl(double s, v3 a) { return mk(s * a.v[0], s * a.v[1], s * a.v[2]); }
static inline v3 dvs(v3 a, double s) { return mk(a.v[0] / s, a.v[1] / s, a.v[2] / s); }
static inline double dot(v3 a, v3 b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }
static inline double nrm(v3 a) { return sqrt(a.v[0] * a.v[0] + a.v[1] * a.v[1] + a.v[2] * a.v[2]); }
static inline v3 crs(v3 a, v3 b) {
    return mk(a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2], a.v[0] * b.v[1] - a.v[1] * b.v[0]);
}
static inline void acc(double* p, v3 a) { p[0] += a.v[0]; p[1] += a.v[1]; p[2] += a.v[2]; }

/* tri::normal_and_area (dA = |n|/2), tri::centroid, tri::signed_volume: fsi/TriangleUtils.h:15-110 */
static void tri_props(v3 v0, v3 v1, v3 v2, double* dA, double* dV, v3* centroid) {
    v3 n = crs(sub(v1, v0), sub(v2, v0));
    double a = nrm(n);
    *dA = a * 0.5;
    *dV = dot(v0, crs(v1, v2)) / 6.;
    *centroid = dvs(add(add(v0, v1), v2), (double)3);
}

/* ------------------------------------------------------------------ shapes */
typedef struct { int64_t i0, i1, t1, t2; double length; } link_t;

static int link_cmp(const void* a, const void* b) {
    const link_t* x = (const link_t*)a;
    const link_t* y = (const link_t*)b;
    if (x->i0 != y->i0) return x->i0 < y->i0 ? -1 : 1;
    if (x->i1 != y->i1) return x->i1 < y->i1 ? -1 : 1;
    return 0;
}

/* ParticleShape constructor + compute_connectivity, fsi/ParticleShape.hh:21-212.
 * Links are unique edges ordered by (min, max) vertex index (the std::set order); every
 * link shared by two triangles gives an adjacent pair whose vertices are permuted so
 * the triangles are (i0,i1,i2) and (i0,i2,i3), with cos/sin of the rest angle.
 * props = [area, volume, cx, cy, cz].  Returns the number of links. */
int64_t orc_shape_connectivity(int64_t nv, const double* xyz, int64_t nt, const int64_t* tri, int64_t* links,
                               double* link_len, int64_t* pairs, double* pair_cs, double* tri_area, double* props,
                               int64_t* npairs_out) {
    (void)nv;
    double area = 0.0, volume = 0.0;
    v3 center = mk(0, 0, 0);
    for (int64_t t = 0; t < nt; ++t) {
        v3 a = ld(xyz + 3 * tri[3 * t]), b = ld(xyz + 3 * tri[3 * t + 1]), c = ld(xyz + 3 * tri[3 * t + 2]);
        v3 n = crs(sub(b, a), sub(c, a));
        double ar = nrm(n);
        ar *= 0.5;
        tri_area[t] = ar;
        area += ar;
        v3 cen = dvs(add(add(a, b), c), (double)3);
        volume += dot(a, crs(b, c)) / 6.;
        center = add(center, scl(ar, cen));
    }
    props[0] = area;
    props[1] = volume;
    center = dvs(center, area);
    props[2] = center.v[0];
    props[3] = center.v[1];
    props[4] = center.v[2];

    link_t* all = (link_t*)malloc(sizeof(link_t) * 3 * (nt > 0 ? nt : 1));
    int64_t na = 0;
    for (int64_t t = 0; t < nt; ++t) {
        int64_t ind[4] = {tri[3 * t], tri[3 * t + 1], tri[3 * t + 2], tri[3 * t]};
        for (int j = 0; j < 3; ++j) {
            link_t l;
            l.i0 = ind[j] < ind[j + 1] ? ind[j] : ind[j + 1];
            l.i1 = ind[j] < ind[j + 1] ? ind[j + 1] : ind[j];
            l.t1 = t;
            l.t2 = -1;
            l.length = nrm(sub(ld(xyz + 3 * l.i0), ld(xyz + 3 * l.i1)));
            all[na++] = l;
        }
    }
    /* stable sort by (i0, i1): the first occurrence of an edge keeps its triangle as t1,
     * a later one becomes t2, as the std::set lookup of compute_connectivity does */
    for (int64_t a = 1; a < na; ++a) {
        link_t key = all[a];
        int64_t b = a - 1;
        while (b >= 0 && (link_cmp(&all[b], &key) > 0)) { all[b + 1] = all[b]; --b; }
        all[b + 1] = key;
    }
    int64_t nl = 0;
    link_t* uniq = (link_t*)malloc(sizeof(link_t) * (na > 0 ? na : 1));
    for (int64_t a = 0; a < na; ++a) {
        if (nl > 0 && uniq[nl - 1].i0 == all[a].i0 && uniq[nl - 1].i1 == all[a].i1) {
            if (uniq[nl - 1].t1 != all[a].t1) uniq[nl - 1].t2 = all[a].t1;
        } else {
            uniq[nl] = all[a];
            uniq[nl].t2 = -1;
            ++nl;
        }
    }
    int64_t np = 0;
    for (int64_t l = 0; l < nl; ++l) {
        links[2 * l] = uniq[l].i0;
        links[2 * l + 1] = uniq[l].i1;
        link_len[l] = uniq[l].length;
        if (uniq[l].t1 < 0 || uniq[l].t2 < 0) continue;
        int64_t a0 = tri[3 * uniq[l].t1], a1 = tri[3 * uniq[l].t1 + 1], a2 = tri[3 * uniq[l].t1 + 2];
        int64_t b0 = tri[3 * uniq[l].t2], b1 = tri[3 * uniq[l].t2 + 1], b2 = tri[3 * uniq[l].t2 + 2];
        const int64_t i0 = uniq[l].i0, i1 = uniq[l].i1;
        /* permute (i0,i1,i2) <- (i2,i0,i1) until the shared edge is (t.i0, t.i2) */
        for (int g = 0; g < 3 && !((a0 == i0 && a2 == i1) || (a0 == i1 && a2 == i0)); ++g) {
            int64_t tmp = a0; a0 = a2; a2 = a1; a1 = tmp;
        }
        /* ... and for the second triangle until it is (t.i0, t.i1) */
        for (int g = 0; g < 3 && !((b0 == i0 && b1 == i1) || (b0 == i1 && b1 == i0)); ++g) {
            int64_t tmp = b0; b0 = b2; b2 = b1; b1 = tmp;
        }
        pairs[4 * np] = a0;
        pairs[4 * np + 1] = a1;
        pairs[4 * np + 2] = a2;
        pairs[4 * np + 3] = b2;
        /* tri::cos_sin_of_angle_between_pair, TriangleUtils.h:125-136 */
        v3 p0 = ld(xyz + 3 * a0), p1 = ld(xyz + 3 * a1), p2 = ld(xyz + 3 * a2), p3 = ld(xyz + 3 * b2);
        v3 n1 = crs(sub(p1, p0), sub(p2, p0));
        n1 = dvs(n1, nrm(n1));
        v3 n2 = crs(sub(p2, p0), sub(p3, p0));
        n2 = dvs(n2, nrm(n2));
        pair_cs[2 * np] = dot(n1, n2);
        pair_cs[2 * np + 1] = ((dot(sub(n1, n2), sub(p1, p3)) > 0) ? 1.0 : -1.0) * nrm(crs(n1, n2));
        ++np;
    }
    free(all);
    free(uniq);
    *npairs_out = np;
    return nl;
}

/* DeformableParticle3D::update, fsi/DeformableParticle3D.hh:54-82.  out = [area, volume, comx, comy, comz] */
void orc_particle_update(int64_t nv, const double* pos, int64_t nt, const int64_t* tri, double* out) {
    (void)nv;
    double area = 0.0, volume = 0.0;
    v3 com = mk(0, 0, 0);
    for (int64_t t = 0; t < nt; ++t) {
        v3 a = ld(pos + 3 * tri[3 * t]), b = ld(pos + 3 * tri[3 * t + 1]), c = ld(pos + 3 * tri[3 * t + 2]);
        v3 cen;
        double dA, dV;
        /* normal_and_area divides the normal by |n| before halving; the area itself is |n|*0.5 */
        tri_props(a, b, c, &dA, &dV, &cen);
        area += dA;
        volume += dV;
        com = add(com, scl(dA, cen));
    }
    com = dvs(com, area);
    out[0] = area;
    out[1] = volume;
    out[2] = com.v[0];
    out[3] = com.v[1];
    out[4] = com.v[2];
}

/* DeformableParticle3D::compute_moment_of_intertia, fsi/DeformableParticle3D.hh:173-272 */
void orc_inertia(const double* pos, int64_t nt, const int64_t* tri, double* I) {
    double in[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t t = 0; t < nt; ++t) {
        const double* v0 = pos + 3 * tri[3 * t];
        const double* v1 = pos + 3 * tri[3 * t + 1];
        const double* v2 = pos + 3 * tri[3 * t + 2];
        v3 N = crs(sub(ld(v1), ld(v0)), sub(ld(v2), ld(v0)));
        double f1[3], f2[3], f3[3], g0[3], g1[3], g2[3];
        for (int d = 0; d < 3; ++d) {
            double tmp0 = v0[d] + v1[d];
            f1[d] = tmp0 + v2[d];
            double tmp1 = v0[d] * v0[d];
            double tmp2 = tmp1 + v1[d] * tmp0;
            f2[d] = tmp2 + v2[d] * f1[d];
            f3[d] = v0[d] * tmp1 + v1[d] * tmp2 + v2[d] * f2[d];
            g0[d] = f2[d] + v0[d] * (f1[d] + v0[d]);
            g1[d] = f2[d] + v1[d] * (f1[d] + v1[d]);
            g2[d] = f2[d] + v2[d] * (f1[d] + v2[d]);
        }
        in[0] += N.v[0] * f1[0];
        in[1] += N.v[0] * f2[0];
        in[2] += N.v[1] * f2[1];
        in[3] += N.v[2] * f2[2];
        in[4] += N.v[0] * f3[0];
        in[5] += N.v[1] * f3[1];
        in[6] += N.v[2] * f3[2];
        in[7] += N.v[0] * (v0[1] * g0[0] + v1[1] * g1[0] + v2[1] * g2[0]);
        in[8] += N.v[1] * (v0[2] * g0[1] + v1[2] * g1[1] + v2[2] * g2[1]);
        in[9] += N.v[2] * (v0[0] * g0[2] + v1[0] * g1[2] + v2[0] * g2[2]);
    }
    const double oneDiv6 = (double)(1.0 / 6.0), oneDiv24 = (double)(1.0 / 24.0);
    const double oneDiv60 = (double)(1.0 / 60.0), oneDiv120 = (double)(1.0 / 120.0);
    in[0] *= oneDiv6;
    in[1] *= oneDiv24; in[2] *= oneDiv24; in[3] *= oneDiv24;
    in[4] *= oneDiv60; in[5] *= oneDiv60; in[6] *= oneDiv60;
    in[7] *= oneDiv120; in[8] *= oneDiv120; in[9] *= oneDiv120;
    const double vol = in[0];
    const double c[3] = {in[1] / vol, in[2] / vol, in[3] / vol};
    I[0] = in[5] + in[6] - vol * (c[1] * c[1] + c[2] * c[2]);
    I[1] = -in[7] + vol * c[0] * c[1];
    I[2] = -in[9] + vol * c[2] * c[0];
    I[3] = I[1];
    I[4] = in[4] + in[6] - vol * (c[2] * c[2] + c[0] * c[0]);
    I[5] = -in[8] + vol * c[1] * c[2];
    I[6] = I[2];
    I[7] = I[5];
    I[8] = in[4] + in[5] - vol * (c[0] * c[0] + c[1] * c[1]);
}

/* ------------------------------------------------------------------ membrane forces */
/* DeformableCapsuleParticle::compute_forces, fsi/DeformableCapsule.hh:60-150, including the
 * reference's deformation-gradient component c = l' sin(phi) / (l' sin(phi0)) (line 96). */
static void capsule_forces(int skalak, double G, double Cc, const double* rest, int64_t nt, const int64_t* tri,
                           const double* tri_area, const double* pos, double* force) {
    for (int64_t t = 0; t < nt; ++t) {
        const int64_t id[3] = {tri[3 * t], tri[3 * t + 1], tri[3 * t + 2]};
        v3 p0 = ld(pos + 3 * id[0]), p1 = ld(pos + 3 * id[1]), p2 = ld(pos + 3 * id[2]);
        v3 e0 = sub(p1, p0), e1 = sub(p2, p0);
        v3 e0_0 = sub(ld(rest + 3 * id[1]), ld(rest + 3 * id[0]));
        v3 e1_0 = sub(ld(rest + 3 * id[2]), ld(rest + 3 * id[0]));
        const double l = nrm(e0), lp = nrm(e1), l0 = nrm(e0_0), l0p = nrm(e1_0);
        const double e0e1 = dot(e0, e1);
        const double sin_phi = nrm(crs(e0, e1)) / (l * lp);
        const double cos_phi = e0e1 / (l * lp);
        const double sin_phi_0 = nrm(crs(e0_0, e1_0)) / (l0 * l0p);
        const double cos_phi_0 = dot(e0_0, e1_0) / (l0 * l0p);
        const double a = l / l0;
        const double b = (lp * cos_phi / l0p - l * cos_phi_0 / l0) / sin_phi_0;
        const double c = lp * sin_phi / (lp * sin_phi_0);
        const double D11 = (a * a - 1.) / 2.;
        const double D22 = (b * b + c * c - 1) / 2.;
        const double D12 = a * b / 2.;
        const double I1 = 2. * (D11 + D22);
        const double I2 = I1 + 4 * (D11 * D22 - D12 * D12);
        v3 gl[3], glp[3], gc[3];
        gl[0] = dvs(e0, -l); gl[1] = dvs(e0, l); gl[2] = mk(0, 0, 0);
        glp[0] = dvs(e1, -lp); glp[1] = mk(0, 0, 0); glp[2] = dvs(e1, lp);
        gc[0] = add(scl(-1. / (l * lp) + e0e1 / (l * l * l * lp), e0), scl(-1. / (l * lp) + e0e1 / (l * lp * lp * lp), e1));
        gc[1] = sub(scl(1. / (l * lp), e1), scl(e0e1 / (l * l * l * lp), e0));
        gc[2] = sub(scl(1. / (l * lp), e0), scl(e0e1 / (l * lp * lp * lp), e1));
        const double s0sq = sin_phi_0 * sin_phi_0;
        for (int i = 0; i < 3; ++i) {
            v3 gD11 = scl(l / (l0 * l0), gl[i]);
            v3 gD22 = scl(1. / s0sq,
                          sub(add(scl(lp / (l0p * l0p) - l * cos_phi * cos_phi_0 / (l0 * l0p), glp[i]),
                                  scl(l * (cos_phi_0 * cos_phi_0) / (l0 * l0) - lp * cos_phi * cos_phi_0 / (l0p * l0), gl[i])),
                              scl(l * lp * cos_phi_0 / (l0 * l0p), gc[i])));
            v3 gD12 = scl(1. / (2. * l0p * sin_phi_0),
                          add(add(scl(lp * cos_phi / l0p - 2. * l * cos_phi_0 / l0, gl[i]), scl(l * cos_phi / l0p, glp[i])),
                              scl(l * lp / l0p, gc[i])));
            v3 gI1 = scl(2., add(gD11, gD22));
            v3 gI2 = sub(add(scl(2. + 4. * D22, gD11), scl(2. + 4. * D11, gD22)), scl(8. * D12, gD12));
            v3 fv;
            if (skalak) {
                fv = scl(-G / 2. * tri_area[t], add(scl(I1 + 1, gI1), scl(Cc * I2 - 1, gI2)));
            } else {
                fv = scl(-G / 2. * tri_area[t], sub(gI1, scl(1. / ((1 + I2) * (1 + I2)), gI2)));
            }
            acc(force + 3 * id[i], fv);
        }
    }
}

/* tri::triangle_area_and_gradient, fsi/TriangleUtils.h:58-103 */
static void area_and_gradient(const double* v0, const double* v1, const double* v2, double* area, v3* g0, v3* g1, v3* g2) {
    const double v01v11 = v0[1] - v1[1], v02v22 = v0[2] - v2[2], v02v12 = v0[2] - v1[2];
    const double v01v21 = v0[1] - v2[1], v00v20 = v0[0] - v2[0], v00v10 = v0[0] - v1[0];
    const double a = v01v11 * v02v22 - v02v12 * v01v21;
    const double b = v02v12 * v00v20 - (v0[0] - v1[0]) * v02v22;
    const double c = v00v10 * v01v21 - v01v11 * v00v20;
    *area = 0.5 * sqrt(a * a + b * b + c * c);
    const double denom = (double)1. / ((double)4. * *area);
    *g0 = mk((b * (v2[2] - v1[2]) + c * (v1[1] - v2[1])) * denom, (a * (v1[2] - v2[2]) + c * (v2[0] - v1[0])) * denom,
             (a * (v2[1] - v1[1]) + b * (v1[0] - v2[0])) * denom);
    *g1 = mk((b * v02v22 + c * (v2[1] - v0[1])) * denom, (a * (v2[2] - v0[2]) + c * v00v20) * denom,
             (a * v01v21 + b * (v2[0] - v0[0])) * denom);
    *g2 = mk((b * (v1[2] - v0[2]) + c * v01v11) * denom, (a * (v02v12) + c * (v1[0] - v0[0])) * denom,
             (a * (v1[1] - v0[1]) + b * v00v10) * denom);
}

/* RBCParameters::in_plane_ks_kp, fsi/RBCParticle.hh:27-44 (x0 = 1/2.2) */
static void in_plane_ks_kp(double G, double l0, double m, double* ks, double* kp) {
    const double x0 = 1. / 2.2;
    const double ks_coeff1 = 0.25 * (6. * x0 + (3 * x0 * x0 - 2 * x0 * x0 * x0) / ((1 - x0) * (1 - x0)));
    const double ks_coeff2 = x0 / (2. * (1 - x0) * (1 - x0) * (1 - x0)) + 0.25 * (1. - 1. / ((1 - x0) * (1 - x0)));
    const double kp_coeff1 = -1. / pow(l0, m);
    const double kp_coeff2 = (m + 1) / pow(l0, m);
    const double G_lhs = (double)4. * l0 * G / sqrt(3.0);
    *ks = -kp_coeff1 * G_lhs / (ks_coeff1 * kp_coeff2 - ks_coeff2 * kp_coeff1);
    *kp = ks_coeff1 * G_lhs / (ks_coeff1 * kp_coeff2 - ks_coeff2 * kp_coeff1);
}

/* RBCParticle::compute_forces, fsi/RBCParticle.hh:140-247 */
static void rbc_forces(const double* prm, int64_t nt, const int64_t* tri, const double* tri_area, double A0,
                       int64_t nl, const int64_t* links, const double* link_len, int64_t np, const int64_t* pairs,
                       const double* pair_cs, const double* pos, double area, double volume, double* force) {
    const double m = 2;
    for (int64_t l = 0; l < nl; ++l) {
        double ks, kp;
        in_plane_ks_kp(prm[ORC_P_SHEAR_MODULUS], link_len[l], m, &ks, &kp);
        const double* p0 = pos + 3 * links[2 * l];
        const double* p1 = pos + 3 * links[2 * l + 1];
        v3 dv = sub(ld(p0), ld(p1));
        const double L = nrm(dv);
        const double x = L / (link_len[l] * 2.2);
        const double df = -0.25 * ks * (6. * x + (3. * x * x - 2. * x * x * x) / ((1 - x) * (1 - x))) + kp / pow(L, m);
        v3 fv = dvs(scl(df, dv), L);
        acc(force + 3 * links[2 * l], fv);
        acc(force + 3 * links[2 * l + 1], scl(-1.0, fv));
    }
    for (int64_t t = 0; t < nt; ++t) {
        const int64_t i0 = tri[3 * t], i1 = tri[3 * t + 1], i2 = tri[3 * t + 2];
        const double *v0 = pos + 3 * i0, *v1 = pos + 3 * i1, *v2 = pos + 3 * i2;
        double la;
        v3 g0, g1, g2;
        area_and_gradient(v0, v1, v2, &la, &g0, &g1, &g2);
        double df_area = 0.;
        df_area += prm[ORC_P_K_AREA_GLOBAL] * (A0 - area) / A0;
        df_area += prm[ORC_P_K_AREA_LOCAL] * (tri_area[t] - la) / tri_area[t];
        acc(force + 3 * i0, scl(df_area, g0));
        acc(force + 3 * i1, scl(df_area, g1));
        acc(force + 3 * i2, scl(df_area, g2));
        /* tri::grad_signed_volume, TriangleUtils.h:113-120 */
        g0 = dvs(crs(ld(v1), ld(v2)), 6.);
        g1 = dvs(crs(ld(v2), ld(v0)), 6.);
        g2 = dvs(crs(ld(v0), ld(v1)), 6.);
        const double df_vol = prm[ORC_P_K_VOLUME] * (prm[ORC_P_VOL_DESIRED] - volume) / prm[ORC_P_VOL_DESIRED];
        acc(force + 3 * i0, scl(df_vol, g0));
        acc(force + 3 * i1, scl(df_vol, g1));
        acc(force + 3 * i2, scl(df_vol, g2));
    }
    for (int64_t p = 0; p < np; ++p) {
        const int64_t* q = pairs + 4 * p;
        v3 v0 = ld(pos + 3 * q[0]), v1 = ld(pos + 3 * q[1]), v2 = ld(pos + 3 * q[2]), v3_ = ld(pos + 3 * q[3]);
        /* tri::grad_angle_between_pair, TriangleUtils.h:139-164 */
        v3 e0 = sub(v1, v0), e1 = sub(v2, v0), e2 = sub(v3_, v0);
        const double e1n = nrm(e1);
        v3 e1u = dvs(e1, e1n);
        v3 n1 = crs(e0, e1), n2 = crs(e1, e2);
        const double n1n = nrm(n1), n2n = nrm(n2);
        v3 n1u = dvs(n1, n1n), n2u = dvs(n2, n2n);
        const double cos_t = dot(n1u, n2u);
        const double sin_t = ((dot(sub(n1, n2), sub(v1, v3_)) > 0) ? (double)1. : (double)-1.) * nrm(crs(n1u, n2u));
        v3 g[4];
        g[0] = add(scl(dot(e1u, sub(e1, e2)) / n2n, n2u), scl(dot(e1u, sub(e1, e0)) / n1n, n1u));
        g[1] = scl(-e1n / n1n, n1u);
        g[2] = add(scl(dot(e1u, e2) / n2n, n2u), scl(dot(e1u, e0) / n1n, n1u));
        g[3] = scl(-e1n / n2n, n2u);
        const double pref = prm[ORC_P_K_BEND] * (-pair_cs[2 * p] * sin_t + pair_cs[2 * p + 1] * cos_t);
        for (int k = 0; k < 4; ++k) acc(force + 3 * q[k], scl(pref, g[k]));
    }
}

/* The element forces added onto `force` (which holds, e.g., the wall-interaction forces the
 * decorators applied first, ImmersedBoundaryDynamics_forces.hh:293-296). */
static void membrane_forces_acc(int32_t model, const double* prm, int64_t nv, const double* rest, int64_t nt,
                                const int64_t* tri, const double* tri_area, double A0, int64_t nl, const int64_t* links,
                                const double* link_len, int64_t np, const int64_t* pairs, const double* pair_cs,
                                const double* pos, double area, double volume, double* force) {
    if (model == ORC_MODEL_CAPSULE_NEOHOOKEAN || model == ORC_MODEL_CAPSULE_SKALAK) {
        capsule_forces(model == ORC_MODEL_CAPSULE_SKALAK, prm[ORC_P_G], prm[ORC_P_C], rest, nt, tri, tri_area, pos, force);
    } else if (model == ORC_MODEL_RBC_WLCPOW) {
        rbc_forces(prm, nt, tri, tri_area, A0, nl, links, link_len, np, pairs, pair_cs, pos, area, volume, force);
    } else {
        /* Skalak in-plane law + the RBC model's area, volume and bending terms; the two are
         * accumulated separately and summed, as a capsule and a zero-shear-modulus RBC
         * evaluated on the same vertices. */
        double* extra = (double*)calloc((size_t)(3 * nv), sizeof(double));
        capsule_forces(1, prm[ORC_P_G], prm[ORC_P_C], rest, nt, tri, tri_area, pos, force);
        double p2[ORC_P_COUNT];
        memcpy(p2, prm, sizeof(p2));
        p2[ORC_P_SHEAR_MODULUS] = 0.0;
        rbc_forces(p2, nt, tri, tri_area, A0, nl, links, link_len, np, pairs, pair_cs, pos, area, volume, extra);
        for (int64_t i = 0; i < 3 * nv; ++i) force[i] += extra[i];
        free(extra);
    }
}

void orc_membrane_forces(int32_t model, const double* prm, int64_t nv, const double* rest, int64_t nt,
                         const int64_t* tri, const double* tri_area, double A0, int64_t nl, const int64_t* links,
                         const double* link_len, int64_t np, const int64_t* pairs, const double* pair_cs,
                         const double* pos, double area, double volume, double* force) {
    memset(force, 0, sizeof(double) * 3 * nv);
    membrane_forces_acc(model, prm, nv, rest, nt, tri, tri_area, A0, nl, links, link_len, np, pairs, pair_cs, pos,
                        area, volume, force);
}

/* ------------------------------------------------------------------ pipe walls */
/* The first-order pipe walls of progs/rbc_in_pipe/rbc_in_pipe.cpp:306-318 on PipeBoundary (axis
 * along x through (y0, z0), fsi/Boundary.h:132-160): BounceBack where the node is not contained
 * ((y - y0)^2 + (z - z0)^2 < radius^2 fails), NoDynamics where it is not contained in the pipe
 * widened by the margin (plint)sqrt(2) = 1. */
void orc_pipe_celltypes(int64_t nx, int64_t ny, int64_t nz, double y0, double z0, double radius, uint8_t* types) {
    const double margin = -(double)(int64_t)sqrt(2.0);
    for (int64_t z = 0; z < nz; ++z)
        for (int64_t y = 0; y < ny; ++y)
            for (int64_t x = 0; x < nx; ++x) {
                const double dy = (double)y - y0, dz = (double)z - z0;
                const double r2 = dy * dy + dz * dz;
                uint8_t t = ORC_CELL_FLUID;
                if (!(r2 < radius * radius)) t = ORC_CELL_BOUNCE_BACK;
                if (!(r2 < (radius - margin) * (radius - margin))) t = ORC_CELL_NO_DYNAMICS;
                types[x + nx * (y + ny * z)] = t;
            }
}

/* PipeBoundary::trace_ray (fsi/Boundary.h:164-187): crossing parameter t in [0, 1] of the
 * segment x0 -> x1 with the cylinder around the x axis through (y0, z0) */
static int pipe_trace_ray(double py0, double pz0, double radius, const double* x0, const double* x1, double* t) {
    const double y1 = x0[1] - py0, y2 = x1[1] - py0, z1 = x0[2] - pz0, z2 = x1[2] - pz0;
    const double a = (y2 - y1) * (y2 - y1) + (z2 - z1) * (z2 - z1);
    const double b = y1 * (y2 - y1) + z1 * (z2 - z1);
    const double c = y1 * y1 + z1 * z1 - radius * radius;
    const double disc = b * b - c * a;
    if (disc < 0. || fabs(a) < 10 * DBL_EPSILON) return 0;
    const double bOverA = -b / a;
    const double sqrtDisc = sqrt(disc) / a;
    *t = bOverA - sqrtDisc;
    if (*t >= 0. && *t <= 1.) return 1;
    *t = bOverA + sqrtDisc;
    if (*t >= 0. && *t <= 1.) return 1;
    return 0;
}

/* GuoRigidWallBoundaryInstantiator::process (fsi/GuoBoundaryCondition.hh:62-130) on a
 * PipeBoundary: every node outside the pipe with a lattice vector that crosses the wall becomes a
 * wall node; among its crossing vectors it keeps the one whose normalised direction has the
 * smallest cosine with the outward normal at pos + dir/|dir| * t, with delta = 1 - t.  Then
 * rbc_in_pipe.cpp:313-318 gives NoDynamics to the nodes outside radius + (plint)sqrt(2). */
int64_t orc_pipe_guo_nodes(int64_t nx, int64_t ny, int64_t nz, double y0, double z0, double radius,
                           orc_guo_node* nodes, uint8_t* types) {
    init_weights();
    const double margin = -(double)(int64_t)sqrt(2.0);
    int64_t count = 0;
    for (int64_t x = 0; x < nx; ++x)
        for (int64_t y = 0; y < ny; ++y)
            for (int64_t z = 0; z < nz; ++z) {
                const double pos[3] = {(double)x, (double)y, (double)z};
                const double dy = pos[1] - y0, dz = pos[2] - z0;
                const int nodyn = !((dy * dy + dz * dz) < (radius - margin) * (radius - margin));
                if (types) types[x + nx * (y + ny * z)] = nodyn ? ORC_CELL_NO_DYNAMICS : ORC_CELL_FLUID;
                if ((dy * dy + dz * dz) < radius * radius) continue;
                double cos_min = 2, delta_min = -1;
                int dir_min = 0, found = 0;
                for (int i = 1; i < Q; ++i) {
                    const double c[3] = {(double)CX[i], (double)CY[i], (double)CZ[i]};
                    const double p2[3] = {pos[0] + c[0], pos[1] + c[1], pos[2] + c[2]};
                    double t = -1;
                    if (!pipe_trace_ray(y0, z0, radius, pos, p2, &t)) continue;
                    const double cn = sqrt((double)(CX[i] * CX[i] + CY[i] * CY[i] + CZ[i] * CZ[i]));
                    const double d2[3] = {c[0] / cn, c[1] / cn, c[2] / cn};
                    const double w[3] = {pos[0] + d2[0] * t, pos[1] + d2[1] * t, pos[2] + d2[2] * t};
                    /* PipeBoundary::get_normal (Boundary.h:245-249) */
                    const double nv[3] = {0, w[1] - y0, w[2] - z0};
                    const double nn = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
                    const double nu[3] = {nv[0] / nn, nv[1] / nn, nv[2] / nn};
                    const double cosang = nu[0] * d2[0] + nu[1] * d2[1] + nu[2] * d2[2];
                    if (cosang < cos_min) {
                        dir_min = i;
                        cos_min = cosang;
                        delta_min = 1 - t;
                    }
                    found = 1;
                }
                if (!found) continue;
                if (nodes) {
                    orc_guo_node* g = &nodes[count];
                    g->x = x, g->y = y, g->z = z;
                    g->dir = dir_min;
                    g->nodyn = nodyn;
                    g->delta = delta_min;
                    g->u[0] = g->u[1] = g->u[2] = 0.0;
                }
                ++count;
            }
    return count;
}

/* GuoRigidWallBoundaryFunctional::process with depth 2 (GuoBoundaryCondition.hh:133-187): the
 * wall node's populations become the equilibrium of the extrapolated wall momentum (with the
 * density of the first fluid node) plus the extrapolated non-equilibrium part of the two fluid
 * nodes along the chosen lattice vector.  A NoDynamics node's equilibrium is 0. */
void orc_apply_guo(const orc_lattice* L, double* f) {
    init_weights();
    const int64_t nx = L->nx, ny = L->ny, nz = L->nz, n = nx * ny * nz;
    for (int64_t g = 0; g < L->nguo; ++g) {
        const orc_guo_node* w = &L->guo[g];
        const int d = w->dir;
        double fc[2][Q], rb[2], j[2][3], fneq[2][Q];
        for (int m = 0; m < 2; ++m) {
            int64_t xs = w->x + (m + 1) * CX[d], ys = w->y + (m + 1) * CY[d], zs = w->z + (m + 1) * CZ[d];
            xs = wrap(xs, nx), ys = wrap(ys, ny), zs = wrap(zs, nz);
            const int64_t k = cell_index(L, xs, ys, zs);
            for (int i = 0; i < Q; ++i) fc[m][i] = f[i * n + k];
            get_rhoBar_j(fc[m], &rb[m], j[m]);
            const double jsq = j[m][0] * j[m][0] + j[m][1] * j[m][1] + j[m][2] * j[m][2];
            const double invRho = (double)1 / (rb[m] + (double)1);
            for (int i = 0; i < Q; ++i) fneq[m][i] = fc[m][i] - bgk_ma2_equilibrium(i, rb[m], invRho, j[m], jsq);
        }
        const double rbw = rb[0];
        double wj[3], jw[3], fw[Q];
        for (int c = 0; c < 3; ++c) wj[c] = (rbw + (double)1) * w->u[c];
        const double dl = w->delta;
        if (dl < (double)0.75) {
            for (int c = 0; c < 3; ++c)
                jw[c] = wj[c] + (dl - (double)1.) * j[0][c] +
                        ((double)1. - dl) / ((double)1. + dl) * ((double)2. * wj[c] + (dl - (double)1.) * j[1][c]);
            for (int i = 0; i < Q; ++i) fw[i] = dl * fneq[0][i] + ((double)1. - dl) * fneq[1][i];
        } else {
            for (int c = 0; c < 3; ++c) jw[c] = (double)1. / dl * (wj[c] + (dl - (double)1.) * j[0][c]);
            for (int i = 0; i < Q; ++i) fw[i] = fneq[0][i];
        }
        const double jsq = jw[0] * jw[0] + jw[1] * jw[1] + jw[2] * jw[2];
        const double invRho = (double)1 / (rbw + (double)1);
        const int64_t k = cell_index(L, w->x, w->y, w->z);
        for (int i = 0; i < Q; ++i)
            f[i * n + k] = (w->nodyn ? 0.0 : bgk_ma2_equilibrium(i, rbw, invRho, jw, jsq)) + fw[i];
    }
}

/* ------------------------------------------------------------------ interaction forces */
/* MorsePotential::eval and SpringPotential::operator() (fsi/Potentials.h:29-71): the force
 * magnitude at distance d, positive = repulsive; both are cut off at r0 (get_cutoff_distance). */
double orc_potential_eval(const orc_potential* p, double d) {
    if (p->kind == ORC_POTENTIAL_MORSE) {
        if (d < 0) d = 0.0;
        const double x = exp(p->beta * (p->r0 - d));
        return 2 * p->beta * p->strength * x * (x - 1);
    }
    if (p->kind == ORC_POTENTIAL_SPRING) return (p->r0 - d) * p->strength;
    return 0.0;
}

/* WallInteraction::apply_force (ForceDecorator.hh:25-32) with ParallelPlatesBoundary(lo, hi) on
 * `axis` (Boundary.h:305-365, plates normal to y there): distance to the nearer plate, outward
 * normal; force -= phi(dist) * normal for dist <= cutoff. */
void orc_wall_forces(const orc_potential* p, int32_t axis, double lo, double hi, int64_t nv, const double* pos,
                     double* force) {
    for (int64_t i = 0; i < nv; ++i) {
        const double r = pos[3 * i + axis];
        const int lower = r < 0.5 * (lo + hi);
        const double dist = lower ? r - lo : hi - r;
        if (dist <= p->r0) {
            const double f = orc_potential_eval(p, dist);
            double n[3] = {0.0, 0.0, 0.0};
            n[axis] = lower ? -1.0 : 1.0;
            for (int d = 0; d < 3; ++d) force[3 * i + d] -= f * n[d];
        }
    }
}

/* WallInteraction on a PipeBoundary along x through (y0, z0) of the given radius
 * (ForceDecorator.hh:25-32; distance_to_boundary and get_normal, Boundary.h:158-161, 245-249):
 * dist = radius - sqrt((y - y0)^2 + (z - z0)^2), force -= phi(dist) (0, dy, dz) / |(0, dy, dz)| */
void orc_pipe_wall_forces(const orc_potential* p, double y0, double z0, double radius, int64_t nv, const double* pos,
                          double* force) {
    for (int64_t i = 0; i < nv; ++i) {
        const double dy = pos[3 * i + 1] - y0, dz = pos[3 * i + 2] - z0;
        const double dist = radius - sqrt(dy * dy + dz * dz);
        if (dist <= p->r0) {
            const double f = orc_potential_eval(p, dist);
            const double nn = sqrt(0.0 * 0.0 + dy * dy + dz * dz);
            const double n[3] = {0.0 / nn, dy / nn, dz / nn};
            for (int d = 0; d < 3; ++d) force[3 * i + d] -= f * n[d];
        }
    }
}

/* Arithmetic1D::min_mod_diff (Periodicity.h:27-35, 96-99) on periodic axes, x - y otherwise */
static double axis_diff(const orc_lattice* L, int a, double x, double y) {
    const int64_t N = a == 0 ? L->nx : (a == 1 ? L->ny : L->nz);
    const double d = x - y;
    if (!L->periodic[a]) return d;
    const double Ld = (double)N, Linv = 1.0 / Ld;
    return d - floor(d * Linv + 0.5) * Ld;
}

/* CollisionHandler::handle_collision (CollisionForces.h:187-199) */
static void pp_pair(const orc_lattice* L, const orc_potential* p, double c2, const double* xa, const double* xb,
                    double* fa, double* fb) {
    const double dr[3] = {axis_diff(L, 0, xb[0], xa[0]), axis_diff(L, 1, xb[1], xa[1]), axis_diff(L, 2, xb[2], xa[2])};
    const double dsq = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
    if (dsq <= c2) {
        const double dist = sqrt(dsq);
        const double s = -orc_potential_eval(p, dist) / dist;
        for (int d = 0; d < 3; ++d) {
            const double df = s * dr[d];
            fa[d] += df;
            fb[d] -= df;
        }
    }
}

/* The domain of a collision grid: the integer bounding box of the lattice (x0..x1 per axis) and
 * its periodic axes (Periodicity3D's arithmetic on that box). */
typedef struct {
    int64_t lo[3], N[3];
    int32_t per[3];
} grid_box;

/* Arithmetic1D::min_mod_diff (Periodicity.h:27-35, 96-99) on periodic axes, x - y otherwise */
static double box_diff(const grid_box* B, int a, double x, double y) {
    const double d = x - y;
    if (!B->per[a]) return d;
    const double Ld = (double)B->N[a], Linv = 1.0 / Ld;
    return d - floor(d * Linv + 0.5) * Ld;
}

/* CollisionHandler::handle_collision (CollisionForces.h:187-199) on a grid box */
static void box_pair(const grid_box* B, const orc_potential* p, double c2, const double* xa, const double* xb,
                     double* fa, double* fb) {
    const double dr[3] = {box_diff(B, 0, xb[0], xa[0]), box_diff(B, 1, xb[1], xa[1]), box_diff(B, 2, xb[2], xa[2])};
    const double dsq = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
    if (dsq <= c2) {
        const double dist = sqrt(dsq);
        const double s = -orc_potential_eval(p, dist) / dist;
        for (int d = 0; d < 3; ++d) {
            const double df = s * dr[d];
            fa[d] += df;
            fb[d] -= df;
        }
    }
}

/* geo::clamp (fsi/geometry.h:20-27) */
static double gclamp(double v, double lo, double hi) { return v >= hi ? hi : (v <= lo ? lo : v); }

/* PipeBoundary::contains(pos, margin) (Boundary.h:148-151) on the (y, z) of a point */
static int pipe_contains(const double* w, double y, double z, double margin) {
    const double dy = y - w[0], dz = z - w[1], r = w[2] - margin;
    return dy * dy + dz * dz < r * r;
}

/* PipeBoundary::does_intersect(rect, width) (Boundary.h:227-243) for a rect's y and z ranges */
static int pipe_does_intersect(const double* w, double ry0, double ry1, double rz0, double rz1, double width) {
    const double cy = w[0] - gclamp(w[0], ry0, ry1), cz = w[1] - gclamp(w[1], rz0, rz1);
    const double tmp = cy * cy + cz * cz;
    if (!(tmp <= w[2] * w[2])) return 0;
    return !(pipe_contains(w, ry0, rz0, width) && pipe_contains(w, ry0, rz1, width) &&
             pipe_contains(w, ry1, rz0, width) && pipe_contains(w, ry1, rz1, width));
}

/* Particle-particle forces as the reference evaluates them
 * (compute_particle_particle_interaction_impl, ImmersedBoundaryDynamics_forces.hh:330-375, with
 * CollisionHandler::compute_collision_forces, CollisionForces.h:63-164, and Grid, Grid.hh):
 * nodes inside the box enlarged by 1/2 + cutoff go into a grid of ~unit cells over the box in
 * particle / vertex order; every bulk cell pairs its nodes among themselves and with the nodes
 * of 7 neighbour cells (+y, +y+z, +z, +x, +x+y, +x+y+z, +x+z), then the first and last bulk
 * layers of each periodic axis are paired.  Pairs whose cells sit at other offsets (e.g. +x-y)
 * are not examined.  With a pipe wall w = {y0, z0, radius} the wall pass follows
 * (CollisionHandler::compute_wall_collision_forces, CollisionForces.h:166-184): every node of a
 * bulk cell the wall intersects (within the cutoff) at distance dist <= cutoff from the wall gets
 * force -= phi(dist) * n, n the outward normal (Boundary.h:158-161, 245-249). */
static void grid_forces(const grid_box* B, const orc_potential* p, int64_t nv, const double* pos,
                        const int32_t* owner, double* force, const double* wall) {
    const double cut = p->r0, c2 = cut * cut;
    double b0[3], b1[3], cs[3], g0[3];
    int64_t nc[3];
    for (int a = 0; a < 3; ++a) {
        b0[a] = (double)B->lo[a] - 0.5;
        b1[a] = (double)(B->lo[a] + B->N[a] - 1) + 0.5 - DBL_EPSILON;
        nc[a] = (int64_t)floor((b1[a] - b0[a]) / 1.0);
        cs[a] = (b1[a] - b0[a]) / (double)nc[a];
        nc[a] += 2;
        g0[a] = b0[a] - cs[a];
    }
    const int64_t ncell = nc[0] * nc[1] * nc[2];
    int64_t* count = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
    int64_t* cell_of = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv > 0 ? nv : 1));
    for (int64_t i = 0; i < nv; ++i) {
        const double* x = pos + 3 * i;
        int in = 1;
        for (int a = 0; a < 3; ++a) in = in && x[a] > b0[a] - cut && x[a] < b1[a] + cut;
        cell_of[i] = -1;
        if (!in) continue;
        int64_t ci[3];
        for (int a = 0; a < 3; ++a) ci[a] = (int64_t)floor((x[a] - g0[a]) / cs[a]);
        cell_of[i] = ci[2] + nc[2] * (ci[1] + nc[1] * ci[0]);
        count[cell_of[i] + 1]++;
    }
    for (int64_t c = 0; c < ncell; ++c) count[c + 1] += count[c];
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncell);
    int64_t* node = (int64_t*)malloc(sizeof(int64_t) * (size_t)(count[ncell] > 0 ? count[ncell] : 1));
    for (int64_t c = 0; c < ncell; ++c) fill[c] = count[c];
    for (int64_t i = 0; i < nv; ++i)
        if (cell_of[i] >= 0) node[fill[cell_of[i]]++] = i;
#define CELL(i, j, k) ((k) + nc[2] * ((j) + nc[1] * (i)))
#define PAIR(u, v)                                                                                     \
    do {                                                                                               \
        const int64_t a_ = (u), b_ = (v);                                                              \
        if (owner[a_] != owner[b_]) box_pair(B, p, c2, pos + 3 * a_, pos + 3 * b_, force + 3 * a_, force + 3 * b_); \
    } while (0)
    for (int64_t i = 1; i <= nc[0] - 2; ++i)
        for (int64_t j = 1; j <= nc[1] - 2; ++j)
            for (int64_t k = 1; k <= nc[2] - 2; ++k) {
                const int64_t c = CELL(i, j, k);
                const int64_t nb[7] = {CELL(i, j + 1, k), CELL(i, j + 1, k + 1), CELL(i, j, k + 1), CELL(i + 1, j, k),
                                       CELL(i + 1, j + 1, k), CELL(i + 1, j + 1, k + 1), CELL(i + 1, j, k + 1)};
                for (int64_t l = count[c]; l < count[c + 1]; ++l) {
                    for (int64_t m = l + 1; m < count[c + 1]; ++m) PAIR(node[l], node[m]);
                    for (int n = 0; n < 7; ++n)
                        for (int64_t m = count[nb[n]]; m < count[nb[n] + 1]; ++m) PAIR(node[l], node[m]);
                }
            }
    /* collide_all_in_cells of the first and last bulk layers of periodic axes (CollisionForces.h:119-163) */
    const int64_t x0 = 1, x1 = nc[0] - 2, y0 = 1, y1 = nc[1] - 2, z0 = 1, z1 = nc[2] - 2;
    const int32_t* per = B->per;
#define ALL(ca, cb)                                                                 \
    do {                                                                            \
        const int64_t p_ = (ca), q_ = (cb);                                         \
        for (int64_t l = count[p_]; l < count[p_ + 1]; ++l)                         \
            for (int64_t m = count[q_]; m < count[q_ + 1]; ++m) PAIR(node[l], node[m]); \
    } while (0)
    if (per[0])
        for (int64_t j = y0; j <= y1; ++j)
            for (int64_t k = z0; k <= z1; ++k) ALL(CELL(x0, j, k), CELL(x1, j, k));
    if (per[1])
        for (int64_t i = x0; i <= x1; ++i)
            for (int64_t k = z0; k <= z1; ++k) ALL(CELL(i, y0, k), CELL(i, y1, k));
    if (per[2])
        for (int64_t i = x0; i <= x1; ++i)
            for (int64_t j = y0; j <= y1; ++j) ALL(CELL(i, j, z0), CELL(i, j, z1));
    if (per[0] && per[1])
        for (int64_t k = z0; k <= z1; ++k) ALL(CELL(x0, y0, k), CELL(x1, y1, k));
    if (per[0] && per[2])
        for (int64_t j = y0; j <= y1; ++j) ALL(CELL(x0, j, z0), CELL(x1, j, z1));
    if (per[1] && per[2])
        for (int64_t i = x0; i <= x1; ++i) ALL(CELL(i, y0, z0), CELL(i, y1, z1));
    if (per[0] && per[1] && per[2]) ALL(CELL(x0, y0, z0), CELL(x1, y1, z1));
    if (wall)
        for (int64_t i = x0; i <= x1; ++i)
            for (int64_t j = y0; j <= y1; ++j)
                for (int64_t k = z0; k <= z1; ++k) {
                    /* the cell's rect: Grid::repartition, Grid.hh:46-58 */
                    const double ry0 = b0[1] + (double)(j - 1) * cs[1], rz0 = b0[2] + (double)(k - 1) * cs[2];
                    if (!pipe_does_intersect(wall, ry0, ry0 + cs[1], rz0, rz0 + cs[2], cut)) continue;
                    const int64_t c = CELL(i, j, k);
                    for (int64_t l = count[c]; l < count[c + 1]; ++l) {
                        const double* x = pos + 3 * node[l];
                        double* f = force + 3 * node[l];
                        const double dy = x[1] - wall[0], dz = x[2] - wall[1];
                        const double dist = wall[2] - sqrt(dy * dy + dz * dz);
                        if (!(dist <= cut)) continue;
                        const double nn = sqrt(0.0 * 0.0 + dy * dy + dz * dz);
                        const double n[3] = {0.0 / nn, dy / nn, dz / nn};
                        const double phi = orc_potential_eval(p, dist);
                        for (int d = 0; d < 3; ++d) f[d] -= phi * n[d];
                    }
                }
#undef ALL
#undef PAIR
#undef CELL
    free(count);
    free(cell_of);
    free(fill);
    free(node);
}

void orc_pp_forces_grid(const orc_lattice* L, const orc_potential* p, int64_t nv, const double* pos,
                        const int32_t* owner, double* force) {
    const grid_box B = {{0, 0, 0}, {L->nx, L->ny, L->nz}, {L->periodic[0], L->periodic[1], L->periodic[2]}};
    grid_forces(&B, p, nv, pos, owner, force, NULL);
}

/* Every pair of vertices of different particles within the cutoff (minimum image on periodic
 * axes), each vertex summing its own terms: for vertex i, the partners j in increasing index
 * order.  This is the interaction the grid search above approximates. */
void orc_pp_forces(const orc_lattice* L, const orc_potential* p, int64_t nv, const double* pos, const int32_t* owner,
                   double* force) {
    const double c2 = p->r0 * p->r0;
    double* acc = (double*)calloc((size_t)(3 * (nv > 0 ? nv : 1)), sizeof(double));
#pragma omp parallel for schedule(dynamic, 64) if (nv > 4096)
    for (int64_t i = 0; i < nv; ++i) {
        double dummy[3];
        for (int64_t j = 0; j < nv; ++j) {
            if (owner[j] == owner[i]) continue;
            pp_pair(L, p, c2, pos + 3 * i, pos + 3 * j, acc + 3 * i, dummy);
        }
    }
    for (int64_t i = 0; i < 3 * nv; ++i) force[i] += acc[i];
    free(acc);
}

/* ------------------------------------------------------------------ growth of the initial distribution */
/* ParticleShape::compute_properties' moment of inertia about the origin (ParticleShape.hh:254-356)
 * and the shape volume, the sum of tri::signed_volume (ParticleShape.hh:21-57, TriangleUtils.h:106-110) */
static void shape_mass_props(int64_t nt, const int64_t* tri, const double* v, double* volume, double* I) {
    double in[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    double vol = 0.0;
    for (int64_t t = 0; t < nt; ++t) {
        const double* v0 = v + 3 * tri[3 * t];
        const double* v1 = v + 3 * tri[3 * t + 1];
        const double* v2 = v + 3 * tri[3 * t + 2];
        const v3 c12 = crs(ld(v1), ld(v2));
        vol += (v0[0] * c12.v[0] + v0[1] * c12.v[1] + v0[2] * c12.v[2]) / 6.;
        const v3 N = crs(sub(ld(v1), ld(v0)), sub(ld(v2), ld(v0)));
        double f1[3], f2[3], f3[3], g0[3], g1[3], g2[3];
        for (int d = 0; d < 3; ++d) {
            const double tmp0 = v0[d] + v1[d];
            f1[d] = tmp0 + v2[d];
            const double tmp1 = v0[d] * v0[d];
            const double tmp2 = tmp1 + v1[d] * tmp0;
            f2[d] = tmp2 + v2[d] * f1[d];
            f3[d] = v0[d] * tmp1 + v1[d] * tmp2 + v2[d] * f2[d];
            g0[d] = f2[d] + v0[d] * (f1[d] + v0[d]);
            g1[d] = f2[d] + v1[d] * (f1[d] + v1[d]);
            g2[d] = f2[d] + v2[d] * (f1[d] + v2[d]);
        }
        in[0] += N.v[0] * f1[0];
        in[1] += N.v[0] * f2[0];
        in[2] += N.v[1] * f2[1];
        in[3] += N.v[2] * f2[2];
        in[4] += N.v[0] * f3[0];
        in[5] += N.v[1] * f3[1];
        in[6] += N.v[2] * f3[2];
        in[7] += N.v[0] * (v0[1] * g0[0] + v1[1] * g1[0] + v2[1] * g2[0]);
        in[8] += N.v[1] * (v0[2] * g0[1] + v1[2] * g1[1] + v2[2] * g2[1]);
        in[9] += N.v[2] * (v0[0] * g0[2] + v1[0] * g1[2] + v2[0] * g2[2]);
    }
    const double oneDiv60 = (double)(1.0 / 60.0), oneDiv120 = (double)(1.0 / 120.0);
    for (int k = 4; k <= 6; ++k) in[k] *= oneDiv60;
    for (int k = 7; k <= 9; ++k) in[k] *= oneDiv120;
    I[0] = in[5] + in[6];
    I[1] = -in[7];
    I[2] = -in[9];
    I[3] = I[1];
    I[4] = in[4] + in[6];
    I[5] = -in[8];
    I[6] = I[2];
    I[7] = I[5];
    I[8] = in[4] + in[5];
    *volume = vol;
}

void orc_shape_mass_props(int64_t nt, const int64_t* tri, const double* xyz, double* volume, double* inertia9) {
    shape_mass_props(nt, tri, xyz, volume, inertia9);
}

/* Quaternion::apply_rotation / apply_inv_rotation (fsi/Quaternion.h:102-146) */
static void q_rotate(const double* q, const double* v, double* r) {
    r[0] = (1 - 2 * (q[2] * q[2] + q[3] * q[3])) * v[0] + 2 * (q[1] * q[2] - q[0] * q[3]) * v[1] +
           2 * (q[0] * q[2] + q[1] * q[3]) * v[2];
    r[1] = 2 * (q[1] * q[2] + q[0] * q[3]) * v[0] + (1 - 2 * (q[1] * q[1] + q[3] * q[3])) * v[1] +
           2 * (q[2] * q[3] - q[0] * q[1]) * v[2];
    r[2] = 2 * (q[1] * q[3] - q[0] * q[2]) * v[0] + 2 * (q[0] * q[1] + q[2] * q[3]) * v[1] +
           (1 - 2 * (q[1] * q[1] + q[2] * q[2])) * v[2];
}
static void q_rotate_inv(const double* q, const double* v, double* r) {
    r[0] = (1 - 2 * (q[2] * q[2] + q[3] * q[3])) * v[0] + 2 * (q[1] * q[2] + q[0] * q[3]) * v[1] +
           2 * (q[1] * q[3] - q[0] * q[2]) * v[2];
    r[1] = 2 * (q[1] * q[2] - q[0] * q[3]) * v[0] + (1 - 2 * (q[1] * q[1] + q[3] * q[3])) * v[1] +
           2 * (q[0] * q[1] + q[2] * q[3]) * v[2];
    r[2] = 2 * (q[0] * q[2] + q[1] * q[3]) * v[0] + 2 * (q[2] * q[3] - q[0] * q[1]) * v[1] +
           (1 - 2 * (q[1] * q[1] + q[2] * q[2])) * v[2];
}
/* Quaternion::to_rot_matrix (Quaternion.h:148-159) */
static void q_matrix(const double* q, double* R) {
    R[0] = 1 - 2 * (q[2] * q[2] + q[3] * q[3]);
    R[1] = 2 * (q[1] * q[2] - q[0] * q[3]);
    R[2] = 2 * (q[0] * q[2] + q[1] * q[3]);
    R[3] = 2 * (q[1] * q[2] + q[0] * q[3]);
    R[4] = 1 - 2 * (q[1] * q[1] + q[3] * q[3]);
    R[5] = 2 * (q[2] * q[3] - q[0] * q[1]);
    R[6] = 2 * (q[1] * q[3] - q[0] * q[2]);
    R[7] = 2 * (q[0] * q[1] + q[2] * q[3]);
    R[8] = 1 - 2 * (q[1] * q[1] + q[2] * q[2]);
}

/* RigidParticle3D::update (RigidParticle.hh:27-36): vertex i at com + R (scale v_i) */
static void rigid_nodes(const double* com, const double* q, double scale, int64_t nv, const double* v, double* pos) {
    double R[9];
    q_matrix(q, R);
    for (int64_t i = 0; i < nv; ++i) {
        const double w[3] = {scale * v[3 * i], scale * v[3 * i + 1], scale * v[3 * i + 2]};
        for (int d = 0; d < 3; ++d) pos[3 * i + d] = com[d] + (R[3 * d] * w[0] + R[3 * d + 1] * w[1] + R[3 * d + 2] * w[2]);
    }
}

/* The growth stage of create_particles (progs/common/create_particles.h:105-161): rigid copies of
 * the shapes (RigidParticle3D, RigidParticle.hh) start at com / quat, every rescale_every
 * iterations are rescaled to initial_scale + (1 - initial_scale) it / n_it, feel
 * compute_collision_forces(SpringPotential(min_dist, strength), &wall) (the collision grid
 * above, the pipe wall when has_wall) and move by RigidParticle3D::move_vertices
 * (RigidParticle.hh:55-101) with the periodic remap of the centre of mass
 * (ImmersedBoundaryDynamics.hh:486-493).  Runs iterations 0 .. it_end - 1 and returns the centres
 * and orientations; pos_out / force_out (optional) receive the vertex positions after the last
 * iteration and the vertex forces of its collision step.  Returns 0, or -1 on bad input. */
int32_t orc_grow_particles(const orc_growth* g, int32_t nshape, const int64_t* nv, const double* verts,
                           const int64_t* nt, const int64_t* tri, int32_t np, const int32_t* shape, double* com,
                           double* quat, double* pos_out, double* force_out) {
    if (nshape < 1 || np < 0 || g->n_it < 1 || g->rescale_every < 1) return -1;
    int64_t* voff = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nshape + 1));
    int64_t* toff = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nshape + 1));
    voff[0] = toff[0] = 0;
    for (int32_t s = 0; s < nshape; ++s) {
        voff[s + 1] = voff[s] + nv[s];
        toff[s + 1] = toff[s] + nt[s];
    }
    double* vol = (double*)malloc(sizeof(double) * (size_t)nshape);
    double* inertia = (double*)malloc(sizeof(double) * 9 * (size_t)nshape);
    for (int32_t s = 0; s < nshape; ++s)
        shape_mass_props(nt[s], tri + 3 * toff[s], verts + 3 * voff[s], &vol[s], inertia + 9 * s);
    int64_t* poff = (int64_t*)malloc(sizeof(int64_t) * (size_t)(np + 1));
    poff[0] = 0;
    for (int32_t p = 0; p < np; ++p) poff[p + 1] = poff[p] + nv[shape[p]];
    const int64_t ntot = poff[np];
    double* pos = (double*)calloc((size_t)(3 * (ntot > 0 ? ntot : 1)), sizeof(double));
    double* frc = (double*)calloc((size_t)(3 * (ntot > 0 ? ntot : 1)), sizeof(double));
    int32_t* owner = (int32_t*)malloc(sizeof(int32_t) * (size_t)(ntot > 0 ? ntot : 1));
    double* vel = (double*)calloc((size_t)(3 * (np > 0 ? np : 1)), sizeof(double));
    double* om = (double*)calloc((size_t)(3 * (np > 0 ? np : 1)), sizeof(double));
    for (int32_t p = 0; p < np; ++p)
        for (int64_t i = poff[p]; i < poff[p + 1]; ++i) owner[i] = p;
    grid_box B;
    for (int a = 0; a < 3; ++a) {
        B.lo[a] = g->box[2 * a];
        B.N[a] = g->box[2 * a + 1] - g->box[2 * a] + 1;
        B.per[a] = g->periodic[a];
    }
    const orc_potential pot = {ORC_POTENTIAL_SPRING, g->min_dist, 0.0, g->strength};
    double scale = g->initial_scale;
    for (int32_t p = 0; p < np; ++p)
        rigid_nodes(com + 3 * p, quat + 4 * p, scale, nv[shape[p]], verts + 3 * voff[shape[p]], pos + 3 * poff[p]);
    for (int64_t it = 0; it < g->it_end; ++it) {
        if (it % g->rescale_every == 0) {
            const double fraction = (double)it / (double)g->n_it;
            scale = g->initial_scale + (1. - g->initial_scale) * fraction;
            for (int32_t p = 0; p < np; ++p)
                rigid_nodes(com + 3 * p, quat + 4 * p, scale, nv[shape[p]], verts + 3 * voff[shape[p]],
                            pos + 3 * poff[p]);
        }
        memset(frc, 0, sizeof(double) * 3 * (size_t)ntot);
        grid_forces(&B, &pot, ntot, pos, owner, frc, g->has_wall ? g->wall : NULL);
        for (int32_t p = 0; p < np; ++p) {
            const int32_t s = shape[p];
            double* c = com + 3 * p;
            double* q = quat + 4 * p;
            double* v = vel + 3 * p;
            double* w = om + 3 * p;
            double F[3] = {0, 0, 0}, Tq[3] = {0, 0, 0};
            for (int64_t i = poff[p]; i < poff[p + 1]; ++i) {
                const double* x = pos + 3 * i;
                const double* f = frc + 3 * i;
                const double r[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
                const double cr[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
                for (int d = 0; d < 3; ++d) {
                    F[d] += f[d];
                    Tq[d] += cr[d];
                }
            }
            double wb[3], Ib[9];
            q_rotate_inv(q, w, wb);
            /* std::pow(T, int) of the reference's C++98 build is __builtin_powi, which g++ expands
             * into the multiplications x^2 = x x, x^3 = x x^2, x^5 = x^2 x^3 */
            const double s2 = scale * scale, s3 = scale * s2, s5 = s2 * s3;
            const double fac = g->density * s5;
            for (int k = 0; k < 9; ++k) Ib[k] = fac * inertia[9 * s + k];
            const double mass = (scale * scale * scale) * vol[s] * g->density;
            double vdot[3];
            for (int d = 0; d < 3; ++d) vdot[d] = F[d] / mass - g->damping * v[d];
            const double Iw[3] = {Ib[0] * wb[0] + Ib[1] * wb[1] + Ib[2] * wb[2], Ib[3] * wb[0] + Ib[4] * wb[1] + Ib[5] * wb[2],
                                  Ib[6] * wb[0] + Ib[7] * wb[1] + Ib[8] * wb[2]};
            const double cw[3] = {wb[1] * Iw[2] - wb[2] * Iw[1], wb[2] * Iw[0] - wb[0] * Iw[2], wb[0] * Iw[1] - wb[1] * Iw[0]};
            double tb[3], rhs[3], sol[3], rw[3];
            q_rotate_inv(q, Tq, tb);
            for (int d = 0; d < 3; ++d) rhs[d] = tb[d] - cw[d];
            /* Matrix<T, 3>::solve (fsi/Matrix3.h:129-144), Cramer's rule */
            const double* m = Ib;
            const double det = m[0] * m[4] * m[8] - m[0] * m[5] * m[7] - m[1] * m[3] * m[8] + m[1] * m[5] * m[6] +
                               m[2] * m[3] * m[7] - m[2] * m[4] * m[6];
            sol[0] = (rhs[2] * (m[1] * m[5] - m[2] * m[4]) + rhs[1] * (m[2] * m[7] - m[1] * m[8]) +
                      rhs[0] * (m[4] * m[8] - m[5] * m[7])) / det;
            sol[1] = (rhs[2] * (m[2] * m[3] - m[0] * m[5]) + rhs[1] * (m[0] * m[8] - m[2] * m[6]) +
                      rhs[0] * (m[5] * m[6] - m[3] * m[8])) / det;
            sol[2] = (rhs[2] * (m[0] * m[4] - m[1] * m[3]) + rhs[1] * (m[1] * m[6] - m[0] * m[7]) +
                      rhs[0] * (m[3] * m[7] - m[4] * m[6])) / det;
            q_rotate(q, sol, rw);
            for (int d = 0; d < 3; ++d) {
                v[d] += vdot[d];
                w[d] += rw[d] - g->damping * w[d];
            }
            for (int d = 0; d < 3; ++d) c[d] += v[d];
            /* unit-norm exponential map (RigidParticle.hh:90-94) */
            const double wn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            if (wn >= (double)10 * DBL_EPSILON) {
                const double ax[3] = {w[0] / wn, w[1] / wn, w[2] / wn};
                const double sh = sin(wn / 2);
                const double r[4] = {cos(wn / 2), sh * ax[0], sh * ax[1], sh * ax[2]};
                const double qn[4] = {r[0] * q[0] - (r[1] * q[1] + r[2] * q[2] + r[3] * q[3]),
                                      r[0] * q[1] + q[0] * r[1] + r[2] * q[3] - r[3] * q[2],
                                      r[0] * q[2] + q[0] * r[2] + r[3] * q[1] - r[1] * q[3],
                                      r[0] * q[3] + q[0] * r[3] + r[1] * q[2] - r[2] * q[1]};
                memcpy(q, qn, sizeof(qn));
            }
            double* px = pos + 3 * poff[p];
            rigid_nodes(c, q, scale, nv[s], verts + 3 * voff[s], px);
            /* map_center_of_mass_to_periodic_grid (ParticleBase.hh:111-136) */
            double np_[3] = {c[0], c[1], c[2]};
            for (int d = 0; d < 3; ++d) {
                if (!B.per[d]) continue;
                const double x0 = (double)B.lo[d] - 0.5, Lf = (double)B.N[d], Linv = 1. / Lf;
                np_[d] = np_[d] - Lf * floor((np_[d] - x0) * Linv);
            }
            const double delta[3] = {np_[0] - c[0], np_[1] - c[1], np_[2] - c[2]};
            for (int64_t i = 0; i < nv[s]; ++i)
                for (int d = 0; d < 3; ++d) px[3 * i + d] += delta[d];
            for (int d = 0; d < 3; ++d) c[d] = np_[d];
        }
    }
    if (pos_out) memcpy(pos_out, pos, sizeof(double) * 3 * (size_t)ntot);
    if (force_out) memcpy(force_out, frc, sizeof(double) * 3 * (size_t)ntot);
    free(voff); free(toff); free(vol); free(inertia); free(poff);
    free(pos); free(frc); free(owner); free(vel); free(om);
    return 0;
}

/* ------------------------------------------------------------------ immersed boundary */
/* RomaDirac<T,3>::eval and PeskinDirac<T,3>::eval(x), fsi/Dirac.h:27-31 and 78-83 */
double orc_dirac(int32_t dirac, double x) {
    if (dirac == ORC_DIRAC_TOPHAT) return 1. - fabs(x); /* TopHatDirac<T,3>::eval, Dirac.h:55-58 */
    const double dx = fabs(x);
    if (dirac == ORC_DIRAC_PESKIN)
        return 0.125 * (dx <= 1 ? (3 - 2 * dx + sqrt(1 + 4 * dx * (1 - dx))) : (5 - 2 * dx - sqrt(-7 + 4 * dx * (3 - dx))));
    return (1.0 / 6.0) * (dx > 0.5 ? (5.0 - 3 * dx - sqrt(-3 * (1 - dx) * (1 - dx) + 1)) : 2.0 * (1 + sqrt(1 - 3 * dx * dx)));
}
static double half_support(int32_t dirac) {
    return dirac == ORC_DIRAC_PESKIN ? 2.0 : (dirac == ORC_DIRAC_TOPHAT ? 1.0 : 1.5);
}
static int support(int32_t dirac) { return dirac == ORC_DIRAC_PESKIN ? 4 : (dirac == ORC_DIRAC_TOPHAT ? 2 : 3); }

/* Arithmetic1D::min_mod_diff for a periodic axis, fsi/Periodicity.h:26-34,93-96 */
static double axis_dist(const orc_lattice* L, int d, double a, double b) {
    const int64_t N = d == 0 ? L->nx : (d == 1 ? L->ny : L->nz);
    if (!L->periodic[d]) return a - b;
    const double Lf = (double)N, Linv = 1. / Lf;
    const double x = a - b;
    return x - floor(x * Linv + 0.5) * Lf;
}

/* geo::Rect::contains(p, arithmetic), fsi/geometry.h:94-100 */
static int rect_contains(const orc_lattice* L, const double* lo, const double* hi, const double* p) {
    for (int d = 0; d < 3; ++d) {
        if (!(fabs(axis_dist(L, d, 0.5 * (lo[d] + hi[d]), p[d])) < 0.5 * (hi[d] - lo[d]))) return 0;
    }
    return 1;
}

/* Node classification of a single-block domain, ImmersedBoundaryDynamics.hh:46-66 and
 * 351-363: 1 = bulk (fast path without range checks), 2 = envelope (general path),
 * 0 = outside the domain and its envelope (no interpolation, no spreading). */
static void classify_pipe(const orc_lattice* L, int32_t dirac, int64_t n, const double* pos, int32_t* cls,
                          const double* pipe);

void orc_classify(const orc_lattice* L, int32_t dirac, int64_t n, const double* pos, int32_t* cls) {
    classify_pipe(L, dirac, n, pos, cls, NULL);
}

/* Node classes (create_nodes_from_particle, ImmersedBoundaryDynamics.hh:345-356): 0 outside the
 * IB envelope, 3 near a pipe boundary (distance_to_boundary_less_than(pos, h + 1), Boundary.h:
 * 154-157), 1 bulk, 2 envelope.  `pipe` = {y0, z0, radius} or NULL. */
static void classify_pipe(const orc_lattice* L, int32_t dirac, int64_t n, const double* pos, int32_t* cls,
                          const double* pipe) {
    const double h = half_support(dirac);
    const double N[3] = {(double)(L->nx - 1), (double)(L->ny - 1), (double)(L->nz - 1)};
    double elo[3], ehi[3], blo[3], bhi[3];
    const double shrink = 0.5 - h - DBL_EPSILON;
    for (int d = 0; d < 3; ++d) {
        elo[d] = 0.0 - h;
        ehi[d] = N[d] + h;
        blo[d] = 0.0 - shrink;
        bhi[d] = N[d] + shrink;
    }
    for (int64_t i = 0; i < n; ++i) {
        const double* p = pos + 3 * i;
        if (!rect_contains(L, elo, ehi, p)) cls[i] = 0;
        else if (pipe && (p[1] - pipe[0]) * (p[1] - pipe[0]) + (p[2] - pipe[1]) * (p[2] - pipe[1]) >
                             (pipe[2] - (h + 1.)) * (pipe[2] - (h + 1.)))
            cls[i] = 3;
        else if (rect_contains(L, blo, bhi, p)) cls[i] = 1;
        else cls[i] = 2;
    }
}

/* Arithmetic1D::remap_int(i, offset) for a periodic axis, Periodicity.h:106-110 (i0 = 0) */
static int64_t remap_index(const orc_lattice* L, int d, int64_t i, int64_t offset) {
    const int64_t N = d == 0 ? L->nx : (d == 1 ? L->ny : L->nz);
    if (!L->periodic[d]) return i;
    int64_t val = ((i + offset + 100 * N) % N) - offset;
    return val < 0 ? val + N : val;
}

static int64_t remap_index(const orc_lattice* L, int d, int64_t i, int64_t offset);

/* GeneralInterpolator::interpolate_node (ImmersedBoundaryDynamics_interpolation.hh:43-78) with
 * any delta kernel: out += sum of the kernel weights times u over the support, nodes outside the
 * lattice skipped */
static void interp_general(const orc_lattice* L, int32_t dirac, int64_t off, const double* u, const double* pr,
                           double* out) {
    const int64_t nn = L->nx * L->ny * L->nz;
    const int64_t nmax[3] = {L->nx, L->ny, L->nz};
    const int s = support(dirac);
    int64_t lo[3];
    for (int d = 0; d < 3; ++d) lo[d] = (int64_t)ceil(pr[d] - half_support(dirac));
    for (int64_t i = lo[0]; i <= lo[0] + s - 1; ++i) {
        const int64_t i2 = remap_index(L, 0, i, off) + off;
        if (i2 < 0 || i2 > nmax[0] - 1) continue;
        const double dxw = orc_dirac(dirac, (double)i - pr[0]);
        for (int64_t j = lo[1]; j <= lo[1] + s - 1; ++j) {
            const int64_t j2 = remap_index(L, 1, j, off) + off;
            if (j2 < 0 || j2 > nmax[1] - 1) continue;
            const double dxy = dxw * orc_dirac(dirac, (double)j - pr[1]);
            for (int64_t kk = lo[2]; kk <= lo[2] + s - 1; ++kk) {
                const int64_t k2 = remap_index(L, 2, kk, off) + off;
                if (k2 < 0 || k2 > nmax[2] - 1) continue;
                const double dxyz = dxy * orc_dirac(dirac, (double)kk - pr[2]);
                const int64_t c = i2 + L->nx * (j2 + L->ny * k2);
                for (int d = 0; d < 3; ++d) out[d] += dxyz * u[d * nn + c];
            }
        }
    }
}

/* GeneralSpreading::spread (ImmersedBoundaryDynamics_forces.hh:52-85) with any delta kernel */
static void spread_general(const orc_lattice* L, int32_t dirac, int64_t off, const double* pr, const double* fv,
                           double* F) {
    const int64_t nn = L->nx * L->ny * L->nz;
    const int64_t nmax[3] = {L->nx, L->ny, L->nz};
    const int s = support(dirac);
    int64_t lo[3];
    for (int d = 0; d < 3; ++d) lo[d] = (int64_t)ceil(pr[d] - half_support(dirac));
    for (int64_t i = lo[0]; i <= lo[0] + s - 1; ++i) {
        const int64_t i2 = remap_index(L, 0, i, off) + off;
        if (i2 < 0 || i2 > nmax[0] - 1) continue;
        const double dxw = orc_dirac(dirac, (double)i - pr[0]);
        for (int64_t j = lo[1]; j <= lo[1] + s - 1; ++j) {
            const int64_t j2 = remap_index(L, 1, j, off) + off;
            if (j2 < 0 || j2 > nmax[1] - 1) continue;
            const double dxy = dxw * orc_dirac(dirac, (double)j - pr[1]);
            for (int64_t kk = lo[2]; kk <= lo[2] + s - 1; ++kk) {
                const int64_t k2 = remap_index(L, 2, kk, off) + off;
                if (k2 < 0 || k2 > nmax[2] - 1) continue;
                const double dxyz = dxy * orc_dirac(dirac, (double)kk - pr[2]);
                const int64_t c = i2 + L->nx * (j2 + L->ny * k2);
                for (int d = 0; d < 3; ++d) F[d * nn + c] += dxyz * fv[d];
            }
        }
    }
}

/* PipeBoundary::distance_to_boundary (Boundary.h:158-161) minus the kernel's half support: the
 * weight of the supplied kernel against the TopHat near the wall */
static double pipe_weight(const double* pipe, const double* p, double h) {
    return pipe[2] - sqrt((p[1] - pipe[0]) * (p[1] - pipe[0]) + (p[2] - pipe[1]) * (p[2] - pipe[1])) - h;
}

/* interpolate_near_boundary (ImmersedBoundaryDynamics_interpolation.hh:181-230): the supplied
 * kernel from h + 1 off the wall on, the TopHat within h, linear in between */
static void interp_near_boundary(const orc_lattice* L, int32_t dirac, double offset, const double* u, const double* p,
                                 const double* pipe, double* out) {
    const double pr[3] = {p[0] - offset, p[1] - offset, p[2] - offset};
    const int64_t off = (int64_t)offset;
    const double weight = pipe_weight(pipe, p, half_support(dirac));
    out[0] = out[1] = out[2] = 0.0;
    if (weight >= 1) {
        interp_general(L, dirac, off, u, pr, out);
    } else if (weight <= 0) {
        interp_general(L, ORC_DIRAC_TOPHAT, off, u, pr, out);
    } else {
        double a[3] = {0.0, 0.0, 0.0};
        interp_general(L, dirac, off, u, pr, a);
        interp_general(L, ORC_DIRAC_TOPHAT, off, u, pr, out);
        for (int d = 0; d < 3; ++d) out[d] = (1. - weight) * out[d] + weight * a[d];
    }
}

/* spread_forces_near_boundary (ImmersedBoundaryDynamics_forces.hh:192-237) */
static void spread_near_boundary(const orc_lattice* L, int32_t dirac, double offset, const double* p, const double* fv,
                                 const double* pipe, double* F) {
    const double pr[3] = {p[0] - offset, p[1] - offset, p[2] - offset};
    const int64_t off = (int64_t)offset;
    const double weight = pipe_weight(pipe, p, half_support(dirac));
    if (weight >= 1) {
        spread_general(L, dirac, off, pr, fv, F);
    } else if (weight <= 0) {
        spread_general(L, ORC_DIRAC_TOPHAT, off, pr, fv, F);
    } else {
        const double fa[3] = {fv[0] * weight, fv[1] * weight, fv[2] * weight};
        const double fb[3] = {fv[0] * (1. - weight), fv[1] * (1. - weight), fv[2] * (1. - weight)};
        spread_general(L, dirac, off, pr, fa, F);
        spread_general(L, ORC_DIRAC_TOPHAT, off, pr, fb, F);
    }
}

/* Interpolation with the data-processor offset convention of the reference: node
 * positions are taken relative to the field's location `offset` (all three axes) and
 * indices are local (global + (-offset)).  In the IB step the velocity field has a
 * one-cell envelope, so offset = -1.
 * Bulk nodes: BulkInterpolator (Roma-specialised formula for Roma, generic loop else),
 * ImmersedBoundaryDynamics_interpolation.hh:84-153; envelope nodes: GeneralInterpolator
 * :43-78.  u is a (3, nz, ny, nx) field. */
static void interpolate_impl(const orc_lattice* L, int32_t dirac, double offset, const double* u, int64_t n,
                             const double* pos, const int32_t* cls, double* vel, const double* pipe) {
    const int64_t nn = L->nx * L->ny * L->nz;
    const double h = half_support(dirac);
    const int s = support(dirac);
    const int64_t off = (int64_t)offset;
    const int64_t nmax[3] = {L->nx, L->ny, L->nz};
    for (int64_t k = 0; k < n; ++k) {
        double* out = vel + 3 * k;
        out[0] = out[1] = out[2] = 0.0;
        if (cls[k] == 0) continue;
        if (cls[k] == 3) {
            interp_near_boundary(L, dirac, offset, u, pos + 3 * k, pipe, out);
            continue;
        }
        const double pr[3] = {pos[3 * k] - offset, pos[3 * k + 1] - offset, pos[3 * k + 2] - offset};
        int64_t lo[3];
        for (int d = 0; d < 3; ++d) lo[d] = (int64_t)ceil(pr[d] - h);
        if (cls[k] == 1 && dirac == ORC_DIRAC_ROMA) {
            double w[3][3];
            for (int d = 0; d < 3; ++d) {
                w[d][0] = orc_dirac(dirac, (double)lo[d] - pr[d]);
                w[d][1] = orc_dirac(dirac, (double)lo[d] + (double)1. - pr[d]);
                w[d][2] = orc_dirac(dirac, (double)(lo[d] + 2) - pr[d]);
            }
            const int64_t i0 = remap_index(L, 0, lo[0], off) + off;
            const int64_t j0 = remap_index(L, 1, lo[1], off) + off;
            const int64_t k0 = remap_index(L, 2, lo[2], off) + off;
            for (int d = 0; d < 3; ++d) {
                const double* ud = u + d * nn;
#define U(a, b, c) ud[(i0 + (a)) + L->nx * ((j0 + (b)) + L->ny * (k0 + (c)))]
                out[d] = w[0][0] * (w[1][0] * (w[2][0] * U(0, 0, 0) + w[2][1] * U(0, 0, 1) + w[2][2] * U(0, 0, 2)) +
                                    w[1][1] * (w[2][0] * U(0, 1, 0) + w[2][1] * U(0, 1, 1) + w[2][2] * U(0, 1, 2)) +
                                    w[1][2] * (w[2][0] * U(0, 2, 0) + w[2][1] * U(0, 2, 1) + w[2][2] * U(0, 2, 2))) +
                         w[0][1] * (w[1][0] * (w[2][0] * U(1, 0, 0) + w[2][1] * U(1, 0, 1) + w[2][2] * U(1, 0, 2)) +
                                    w[1][1] * (w[2][0] * U(1, 1, 0) + w[2][1] * U(1, 1, 1) + w[2][2] * U(1, 1, 2)) +
                                    w[1][2] * (w[2][0] * U(1, 2, 0) + w[2][1] * U(1, 2, 1) + w[2][2] * U(1, 2, 2))) +
                         w[0][2] * (w[1][0] * (w[2][0] * U(2, 0, 0) + w[2][1] * U(2, 0, 1) + w[2][2] * U(2, 0, 2)) +
                                    w[1][1] * (w[2][0] * U(2, 1, 0) + w[2][1] * U(2, 1, 1) + w[2][2] * U(2, 1, 2)) +
                                    w[1][2] * (w[2][0] * U(2, 2, 0) + w[2][1] * U(2, 2, 1) + w[2][2] * U(2, 2, 2)));
#undef U
            }
            continue;
        }
        const int general = cls[k] == 2;
        for (int64_t i = lo[0]; i <= lo[0] + s - 1; ++i) {
            const int64_t i2 = remap_index(L, 0, i, off) + off;
            if (general && (i2 < 0 || i2 > nmax[0] - 1)) continue;
            const double dxw = orc_dirac(dirac, (double)i - pr[0]);
            for (int64_t j = lo[1]; j <= lo[1] + s - 1; ++j) {
                const int64_t j2 = remap_index(L, 1, j, off) + off;
                if (general && (j2 < 0 || j2 > nmax[1] - 1)) continue;
                const double dxy = dxw * orc_dirac(dirac, (double)j - pr[1]);
                for (int64_t kk = lo[2]; kk <= lo[2] + s - 1; ++kk) {
                    const int64_t k2 = remap_index(L, 2, kk, off) + off;
                    if (general && (k2 < 0 || k2 > nmax[2] - 1)) continue;
                    const double dxyz = dxy * orc_dirac(dirac, (double)kk - pr[2]);
                    const int64_t c = i2 + L->nx * (j2 + L->ny * k2);
                    for (int d = 0; d < 3; ++d) out[d] += dxyz * u[d * nn + c];
                }
            }
        }
    }
}

/* Spreading: bulk nodes first (BulkSpreading, Roma-specialised for Roma), then the
 * envelope nodes (GeneralSpreading), as compute_and_spread_forces orders them,
 * ImmersedBoundaryDynamics_forces.hh:22-163 and 243-284.  F is (3, nz, ny, nx). */
void orc_interpolate(const orc_lattice* L, int32_t dirac, double offset, const double* u, int64_t n,
                     const double* pos, const int32_t* cls, double* vel) {
    interpolate_impl(L, dirac, offset, u, n, pos, cls, vel, NULL);
}

static void spread_impl(const orc_lattice* L, int32_t dirac, double offset, int64_t n, const double* pos,
                        const double* force, const int32_t* cls, double* F, const double* pipe) {
    const int64_t nn = L->nx * L->ny * L->nz;
    const double h = half_support(dirac);
    const int s = support(dirac);
    const int64_t off = (int64_t)offset;
    const int64_t nmax[3] = {L->nx, L->ny, L->nz};
    for (int pass = 1; pass <= 2; ++pass) {
        for (int64_t k = 0; k < n; ++k) {
            if (cls[k] != pass) continue;
            const double pr[3] = {pos[3 * k] - offset, pos[3 * k + 1] - offset, pos[3 * k + 2] - offset};
            const double* fv = force + 3 * k;
            int64_t lo[3];
            for (int d = 0; d < 3; ++d) lo[d] = (int64_t)ceil(pr[d] - h);
            if (pass == 1 && dirac == ORC_DIRAC_ROMA) {
                double w[3][3];
                for (int d = 0; d < 3; ++d) {
                    w[d][0] = orc_dirac(dirac, (double)lo[d] - pr[d]);
                    w[d][1] = orc_dirac(dirac, (double)lo[d] + (double)1. - pr[d]);
                    w[d][2] = orc_dirac(dirac, (double)(lo[d] + 2) - pr[d]);
                }
                const int64_t i0 = remap_index(L, 0, lo[0], off) + off;
                const int64_t j0 = remap_index(L, 1, lo[1], off) + off;
                const int64_t k0 = remap_index(L, 2, lo[2], off) + off;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        for (int c = 0; c < 3; ++c) {
                            const double wt = w[0][a] * w[1][b] * w[2][c];
                            const int64_t cell = (i0 + a) + L->nx * ((j0 + b) + L->ny * (k0 + c));
                            for (int d = 0; d < 3; ++d) F[d * nn + cell] += wt * fv[d];
                        }
                continue;
            }
            const int general = pass == 2;
            for (int64_t i = lo[0]; i <= lo[0] + s - 1; ++i) {
                const int64_t i2 = remap_index(L, 0, i, off) + off;
                if (general && (i2 < 0 || i2 > nmax[0] - 1)) continue;
                const double dxw = orc_dirac(dirac, (double)i - pr[0]);
                for (int64_t j = lo[1]; j <= lo[1] + s - 1; ++j) {
                    const int64_t j2 = remap_index(L, 1, j, off) + off;
                    if (general && (j2 < 0 || j2 > nmax[1] - 1)) continue;
                    const double dxy = dxw * orc_dirac(dirac, (double)j - pr[1]);
                    for (int64_t kk = lo[2]; kk <= lo[2] + s - 1; ++kk) {
                        const int64_t k2 = remap_index(L, 2, kk, off) + off;
                        if (general && (k2 < 0 || k2 > nmax[2] - 1)) continue;
                        const double dxyz = dxy * orc_dirac(dirac, (double)kk - pr[2]);
                        const int64_t c = i2 + L->nx * (j2 + L->ny * k2);
                        for (int d = 0; d < 3; ++d) F[d * nn + c] += dxyz * fv[d];
                    }
                }
            }
        }
    }    /* the nodes near a boundary last (compute_and_spread_forces, _forces.hh:277-282) */
    for (int64_t k = 0; k < n; ++k)
        if (cls[k] == 3) spread_near_boundary(L, dirac, offset, pos + 3 * k, force + 3 * k, pipe, F);
}

void orc_spread(const orc_lattice* L, int32_t dirac, double offset, int64_t n, const double* pos,
                const double* force, const int32_t* cls, double* F) {
    spread_impl(L, dirac, offset, n, pos, force, cls, F, NULL);
}

int32_t orc_threads(void) {
#ifdef _OPENMP
    return (int32_t)omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ coupled system */
typedef struct {
    int64_t nv, nt, nl, np;
    double *rest, *tri_area, *link_len, *pair_cs;
    int64_t *tri, *links, *pairs;
    double area, volume;
} orc_shape;

typedef struct {
    int32_t shape, model;
    double prm[ORC_P_COUNT];
    double *pos, *vel, *force;
    double area, volume, com[3];
} orc_particle;

struct orc_sys {
    orc_lattice L;
    int32_t dirac;
    double offset;
    double body[3];
    double *f, *ftmp, *F, *phase, *u;
    orc_shape* shapes;
    int32_t nshapes;
    orc_particle* parts;
    int32_t nparts;
    int32_t* cls;
    int64_t ncls;
    int32_t voxelize;
    /* force decorators (wall interactions) and particle-particle interactions */
    int32_t nwalls;
    orc_potential wall_pot[8];
    int32_t wall_axis[8];
    double wall_lo[8], wall_hi[8], wall_r[8]; /* axis 3: a pipe along x, (lo, hi) = (y0, z0), radius r */
    int32_t npp;
    orc_potential pp_pot[8];
    int32_t pp_grid;  /* 1: the reference's grid search, 0: every pair within the cutoff */
    int32_t has_pipe; /* a PipeBoundary set with set_boundary */
    double pipe[3];   /* y0, z0, radius */
};

orc_sys* orc_sys_create(const orc_lattice* L, int32_t dirac, double ib_offset) {
    init_weights();
    orc_sys* s = (orc_sys*)calloc(1, sizeof(orc_sys));
    s->L = *L;
    s->dirac = dirac;
    s->offset = ib_offset;
    const int64_t n = L->nx * L->ny * L->nz;
    s->f = (double*)calloc((size_t)(Q * n), sizeof(double));
    s->ftmp = (double*)calloc((size_t)(Q * n), sizeof(double));
    s->F = (double*)calloc((size_t)(3 * n), sizeof(double));
    s->phase = (double*)calloc((size_t)n, sizeof(double));
    s->u = (double*)calloc((size_t)(3 * n), sizeof(double));
    return s;
}

void orc_sys_destroy(orc_sys* s) {
    if (!s) return;
    for (int32_t i = 0; i < s->nshapes; ++i) {
        orc_shape* sh = &s->shapes[i];
        free(sh->rest); free(sh->tri_area); free(sh->link_len); free(sh->pair_cs);
        free(sh->tri); free(sh->links); free(sh->pairs);
    }
    for (int32_t i = 0; i < s->nparts; ++i) {
        free(s->parts[i].pos); free(s->parts[i].vel); free(s->parts[i].force);
    }
    free(s->shapes); free(s->parts); free(s->cls);
    free(s->f); free(s->ftmp); free(s->F); free(s->phase); free(s->u);
    free(s);
}

double* orc_sys_f(orc_sys* s) { return s->f; }
double* orc_sys_force(orc_sys* s) { return s->F; }
double* orc_sys_phase(orc_sys* s) { return s->phase; }
void orc_sys_set_body_force(orc_sys* s, const double* b) { s->body[0] = b[0]; s->body[1] = b[1]; s->body[2] = b[2]; }

int32_t orc_sys_add_shape(orc_sys* s, int64_t nv, const double* xyz, int64_t nt, const int64_t* tri) {
    s->shapes = (orc_shape*)realloc(s->shapes, sizeof(orc_shape) * (size_t)(s->nshapes + 1));
    orc_shape* sh = &s->shapes[s->nshapes];
    memset(sh, 0, sizeof(*sh));
    sh->nv = nv;
    sh->nt = nt;
    sh->rest = (double*)malloc(sizeof(double) * 3 * nv);
    memcpy(sh->rest, xyz, sizeof(double) * 3 * nv);
    sh->tri = (int64_t*)malloc(sizeof(int64_t) * 3 * nt);
    memcpy(sh->tri, tri, sizeof(int64_t) * 3 * nt);
    sh->tri_area = (double*)malloc(sizeof(double) * nt);
    sh->links = (int64_t*)malloc(sizeof(int64_t) * 6 * nt);
    sh->link_len = (double*)malloc(sizeof(double) * 3 * nt);
    sh->pairs = (int64_t*)malloc(sizeof(int64_t) * 12 * nt);
    sh->pair_cs = (double*)malloc(sizeof(double) * 6 * nt);
    double props[5];
    sh->nl = orc_shape_connectivity(nv, xyz, nt, tri, sh->links, sh->link_len, sh->pairs, sh->pair_cs, sh->tri_area,
                                    props, &sh->np);
    sh->area = props[0];
    sh->volume = props[1];
    return s->nshapes++;
}

static void particle_refresh(orc_sys* s, orc_particle* p) {
    const orc_shape* sh = &s->shapes[p->shape];
    double st[5];
    orc_particle_update(sh->nv, p->pos, sh->nt, sh->tri, st);
    p->area = st[0];
    p->volume = st[1];
    p->com[0] = st[2]; p->com[1] = st[3]; p->com[2] = st[4];
}

/* ParticleBase3D::map_center_of_mass_to_periodic_grid + set_center_of_mass,
 * fsi/ParticleBase.hh:111-136 with Arithmetic1D::remap_pos (Periodicity.h:80-85). */
static void remap_com(orc_sys* s, orc_particle* p) {
    const orc_shape* sh = &s->shapes[p->shape];
    double np_[3] = {p->com[0], p->com[1], p->com[2]};
    const int64_t N[3] = {s->L.nx, s->L.ny, s->L.nz};
    for (int d = 0; d < 3; ++d) {
        if (!s->L.periodic[d]) continue;
        const double x0 = (double)0 - 0.5, Lf = (double)N[d], Linv = 1. / Lf;
        np_[d] = np_[d] - Lf * floor((np_[d] - x0) * Linv);
    }
    const double delta[3] = {np_[0] - p->com[0], np_[1] - p->com[1], np_[2] - p->com[2]};
    for (int64_t i = 0; i < sh->nv; ++i)
        for (int d = 0; d < 3; ++d) p->pos[3 * i + d] += delta[d];
    p->com[0] = np_[0]; p->com[1] = np_[1]; p->com[2] = np_[2];
}

int32_t orc_sys_add_particle(orc_sys* s, int32_t shape, int32_t model, const double* prm, const double* pos) {
    s->parts = (orc_particle*)realloc(s->parts, sizeof(orc_particle) * (size_t)(s->nparts + 1));
    orc_particle* p = &s->parts[s->nparts];
    memset(p, 0, sizeof(*p));
    const orc_shape* sh = &s->shapes[shape];
    p->shape = shape;
    p->model = model;
    memcpy(p->prm, prm, sizeof(p->prm));
    p->pos = (double*)malloc(sizeof(double) * 3 * sh->nv);
    p->vel = (double*)calloc((size_t)(3 * sh->nv), sizeof(double));
    p->force = (double*)calloc((size_t)(3 * sh->nv), sizeof(double));
    memcpy(p->pos, pos ? pos : sh->rest, sizeof(double) * 3 * sh->nv);
    particle_refresh(s, p);
    remap_com(s, p); /* add_particle maps the copy's centre of mass, ImmersedBoundaryDynamics.hh:514-520 */
    return s->nparts++;
}

static void gather_vertices(orc_sys* s, double** pos, int64_t* ntot);

/* all particles' triangles with global vertex indices, then the voxelization */
static void sys_voxelize(orc_sys* s) {
    if (!s->voxelize || s->nparts == 0) return;
    double* pos;
    int64_t nvt, ntt = 0;
    gather_vertices(s, &pos, &nvt);
    for (int32_t i = 0; i < s->nparts; ++i) ntt += s->shapes[s->parts[i].shape].nt;
    int64_t* tri = (int64_t*)malloc(sizeof(int64_t) * 3 * (size_t)(ntt > 0 ? ntt : 1));
    int64_t t = 0, vo = 0;
    for (int32_t i = 0; i < s->nparts; ++i) {
        const orc_shape* sh = &s->shapes[s->parts[i].shape];
        for (int64_t k = 0; k < sh->nt; ++k, ++t)
            for (int c = 0; c < 3; ++c) tri[3 * t + c] = vo + sh->tri[3 * k + c];
        vo += sh->nv;
    }
    orc_voxelize(&s->L, nvt, pos, ntt, tri, s->phase);
    free(pos);
    free(tri);
}

void orc_sys_set_voxelize(orc_sys* s, int32_t on) { s->voxelize = on; }

int32_t orc_sys_add_pipe_wall_interaction(orc_sys* s, const orc_potential* p, double y0, double z0, double radius) {
    if (s->nwalls >= 8 || !(radius > 0)) return -1;
    s->wall_pot[s->nwalls] = *p;
    s->wall_axis[s->nwalls] = 3;
    s->wall_lo[s->nwalls] = y0;
    s->wall_hi[s->nwalls] = z0;
    s->wall_r[s->nwalls] = radius;
    return s->nwalls++;
}

int32_t orc_sys_add_wall_interaction(orc_sys* s, const orc_potential* p, int32_t axis, double lo, double hi) {
    if (s->nwalls >= 8 || axis < 0 || axis > 2) return -1;
    s->wall_r[s->nwalls] = 0.0;
    s->wall_pot[s->nwalls] = *p;
    s->wall_axis[s->nwalls] = axis;
    s->wall_lo[s->nwalls] = lo;
    s->wall_hi[s->nwalls] = hi;
    return s->nwalls++;
}

/* DeformableParticle3D::move_vertices (DeformableParticle3D.hh:26-51): explicit Euler; with a
 * pipe boundary a step that crosses the wall is reflected about the normal at the crossing */
void orc_move_vertices(int64_t nv, double* pos, const double* vel, const double* pipe) {
    for (int64_t v = 0; v < nv; ++v) {
        double* x = pos + 3 * v;
        const double* u = vel + 3 * v;
        const double old[3] = {x[0], x[1], x[2]};
        for (int d = 0; d < 3; ++d) x[d] += u[d];
        double t;
        if (pipe && pipe_trace_ray(pipe[0], pipe[1], pipe[2], old, x, &t)) {
            for (int d = 0; d < 3; ++d) x[d] = old[d] + t * u[d];
            const double nv0[3] = {0, x[1] - pipe[0], x[2] - pipe[1]};
            const double nn = sqrt(nv0[0] * nv0[0] + nv0[1] * nv0[1] + nv0[2] * nv0[2]);
            const double nrm_[3] = {nv0[0] / nn, nv0[1] / nn, nv0[2] / nn};
            const double dt2 = 2. * (u[0] * nrm_[0] + u[1] * nrm_[1] + u[2] * nrm_[2]);
            for (int d = 0; d < 3; ++d) x[d] += (u[d] - dt2 * nrm_[d]) * (1. - t);
        }
    }
}

void orc_sys_set_pipe(orc_sys* s, double y0, double z0, double radius) {
    s->has_pipe = 1;
    s->pipe[0] = y0, s->pipe[1] = z0, s->pipe[2] = radius;
}

int32_t orc_sys_add_pp_interaction(orc_sys* s, const orc_potential* p, int32_t grid) {
    if (s->npp >= 8) return -1;
    s->pp_pot[s->npp] = *p;
    s->pp_grid = grid;
    return s->npp++;
}

/* ImmersedBoundaryDynamics3D::init voxelizes the initial positions (ImmersedBoundaryDynamics.hh:404-412) */
void orc_sys_init(orc_sys* s) { sys_voxelize(s); }

static void gather_vertices(orc_sys* s, double** pos, int64_t* ntot) {
    int64_t n = 0;
    for (int32_t i = 0; i < s->nparts; ++i) n += s->shapes[s->parts[i].shape].nv;
    *ntot = n;
    *pos = (double*)malloc(sizeof(double) * 3 * (n > 0 ? n : 1));
    int64_t o = 0;
    for (int32_t i = 0; i < s->nparts; ++i) {
        const int64_t nv = s->shapes[s->parts[i].shape].nv;
        memcpy(*pos + 3 * o, s->parts[i].pos, sizeof(double) * 3 * nv);
        o += nv;
    }
}

/* One coupled step in the driver order of progs/capsule_in_shear/capsule_in_shear.cpp:187-227:
 * computeVelocity -> setExternalVector(body) -> IB step (interpolate, compute + spread forces,
 * move, update) -> collideAndStream (+ wall processors). */
static void sys_step(orc_sys* s) {
    const orc_lattice* L = &s->L;
    const int64_t n = L->nx * L->ny * L->nz;
    orc_compute_velocity(L, s->f, s->F, s->u);
    for (int d = 0; d < 3; ++d) {
        const double b = s->body[d];
        double* Fd = s->F + d * n;
#pragma omp parallel for schedule(static) if (n > 262144)
        for (int64_t k = 0; k < n; ++k) Fd[k] = b;
    }
    if (s->nparts > 0) {
        double* pos;
        int64_t nvt;
        gather_vertices(s, &pos, &nvt);
        int32_t* cls = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nvt > 0 ? nvt : 1));
        double* vel = (double*)malloc(sizeof(double) * 3 * (nvt > 0 ? nvt : 1));
        double* frc = (double*)malloc(sizeof(double) * 3 * (nvt > 0 ? nvt : 1));
        const double* pipe = s->has_pipe ? s->pipe : NULL;
        classify_pipe(L, s->dirac, nvt, pos, cls, pipe);
        interpolate_impl(L, s->dirac, s->offset, s->u, nvt, pos, cls, vel, pipe);
        int64_t o = 0;
        for (int32_t i = 0; i < s->nparts; ++i) {
            orc_particle* p = &s->parts[i];
            const orc_shape* sh = &s->shapes[p->shape];
            /* ImmersedBoundaryDynamics3D::compute_forces (ImmersedBoundaryDynamics_forces.hh:287-302):
             * zero, the force decorators, then the particle's own forces */
            memset(p->force, 0, sizeof(double) * 3 * sh->nv);
            for (int32_t w = 0; w < s->nwalls; ++w) {
                if (s->wall_axis[w] == 3)
                    orc_pipe_wall_forces(&s->wall_pot[w], s->wall_lo[w], s->wall_hi[w], s->wall_r[w], sh->nv, p->pos,
                                         p->force);
                else
                    orc_wall_forces(&s->wall_pot[w], s->wall_axis[w], s->wall_lo[w], s->wall_hi[w], sh->nv, p->pos,
                                    p->force);
            }
            membrane_forces_acc(p->model, p->prm, sh->nv, sh->rest, sh->nt, sh->tri, sh->tri_area, sh->area, sh->nl,
                                sh->links, sh->link_len, sh->np, sh->pairs, sh->pair_cs, p->pos, p->area, p->volume,
                                p->force);
            memcpy(p->vel, vel + 3 * o, sizeof(double) * 3 * sh->nv);
            memcpy(frc + 3 * o, p->force, sizeof(double) * 3 * sh->nv);
            o += sh->nv;
        }
        if (s->npp > 0) {  /* then the particle-particle interactions over all vertices */
            int32_t* owner = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nvt > 0 ? nvt : 1));
            int64_t q = 0;
            for (int32_t i = 0; i < s->nparts; ++i)
                for (int64_t k = 0; k < s->shapes[s->parts[i].shape].nv; ++k) owner[q++] = i;
            for (int32_t k = 0; k < s->npp; ++k) {
                if (s->pp_grid) orc_pp_forces_grid(L, &s->pp_pot[k], nvt, pos, owner, frc);
                else orc_pp_forces(L, &s->pp_pot[k], nvt, pos, owner, frc);
            }
            q = 0;
            for (int32_t i = 0; i < s->nparts; ++i) {
                const int64_t nvi = s->shapes[s->parts[i].shape].nv;
                memcpy(s->parts[i].force, frc + 3 * q, sizeof(double) * 3 * nvi);
                q += nvi;
            }
            free(owner);
        }
        spread_impl(L, s->dirac, s->offset, nvt, pos, frc, cls, s->F, pipe);
        for (int32_t i = 0; i < s->nparts; ++i) {
            orc_particle* p = &s->parts[i];
            const orc_shape* sh = &s->shapes[p->shape];
            orc_move_vertices(sh->nv, p->pos, p->vel, pipe);
            particle_refresh(s, p);
            remap_com(s, p);
        }
        free(pos); free(cls); free(vel); free(frc);
        /* move_vertices_and_revoxelize, ImmersedBoundaryDynamics.hh:461-483 */
        sys_voxelize(s);
    }
    orc_collide_stream(L, s->f, s->ftmp, s->F, s->phase);
}

void orc_sys_step(orc_sys* s, int64_t nsteps) {
    for (int64_t i = 0; i < nsteps; ++i) sys_step(s);
}

void orc_sys_lattice_only_step(orc_sys* s, int64_t nsteps) {
    for (int64_t i = 0; i < nsteps; ++i) orc_collide_stream(&s->L, s->f, s->ftmp, s->F, s->phase);
}

void orc_sys_get_particle(orc_sys* s, int32_t pid, double* pos, double* vel, double* force, double* stats) {
    orc_particle* p = &s->parts[pid];
    const int64_t nv = s->shapes[p->shape].nv;
    if (pos) memcpy(pos, p->pos, sizeof(double) * 3 * nv);
    if (vel) memcpy(vel, p->vel, sizeof(double) * 3 * nv);
    if (force) memcpy(force, p->force, sizeof(double) * 3 * nv);
    if (stats) {
        stats[0] = p->area; stats[1] = p->volume;
        stats[2] = p->com[0]; stats[3] = p->com[1]; stats[4] = p->com[2];
    }
}

void orc_sys_velocity(orc_sys* s, double* u) { orc_compute_velocity(&s->L, s->f, s->F, u); }

/* ------------------------------------------------------------------ RBC shape calibration */
/* shrink_rbc_volume (progs/common/calibrate_rbc_shape.h:12-69) of an RBCParticle built on a shape
 * (positions = the shape's vertices, area / volume = the shape's, zero velocities): the forces
 * are computed once, then each iteration it = 0 .. 2 n_it sets vol_desired = V0 + it/n_it
 * (vol_final - V0) while it <= n_it and runs RBCParticle::relax_nodes (RBCParticle.hh:318-342):
 * node masses M_i = sum over the triangles at i of area/3 (in triangle order), vel += force/M -
 * damping vel, pos += vel, update (area, volume), forces of the new positions.  An area that
 * turns NaN restarts the whole relaxation with the damping doubled (64 times at most, then -1
 * is returned: the reference would retry forever).  Returns the damping used;
 * pos (3 nv) receives the relaxed vertices, vel (3 nv, optional) their velocities. */
double orc_rbc_shrink_volume(const double* prm_in, int64_t nv, const double* rest, int64_t nt, const int64_t* tri,
                             const double* tri_area, double A0, double V0, int64_t nl, const int64_t* links,
                             const double* link_len, int64_t np, const int64_t* pairs, const double* pair_cs,
                             double vol_final, int64_t n_it, double damping, double* pos, double* vel_out) {
    double* F0 = (double*)calloc(3 * nv, sizeof(double));
    double* F = (double*)malloc(sizeof(double) * 3 * nv);
    double* vel = (double*)malloc(sizeof(double) * 3 * nv);
    double* M = (double*)malloc(sizeof(double) * nv);
    double prm[ORC_P_COUNT];
    orc_membrane_forces(ORC_MODEL_RBC_WLCPOW, prm_in, nv, rest, nt, tri, tri_area, A0, nl, links, link_len, np, pairs,
                        pair_cs, rest, A0, V0, F0);
    for (int attempt = 0;; ++attempt) {
        if (attempt == 64) { /* the reference retries forever; this restatement gives up like the product */
            damping = -1.0;
            break;
        }
        memcpy(pos, rest, sizeof(double) * 3 * nv);
        memcpy(F, F0, sizeof(double) * 3 * nv);
        memset(vel, 0, sizeof(double) * 3 * nv);
        memcpy(prm, prm_in, sizeof(prm));
        int success = 1;
        for (int64_t it = 0;; ++it) {
            if (it <= n_it) prm[ORC_P_VOL_DESIRED] = V0 + ((double)it / (double)n_it) * (vol_final - V0);
            for (int64_t i = 0; i < nv; ++i) M[i] = 0.0;
            for (int64_t t = 0; t < nt; ++t) {
                const int64_t i0 = tri[3 * t], i1 = tri[3 * t + 1], i2 = tri[3 * t + 2];
                const v3 a = ld(pos + 3 * i0);
                const double la = 0.5 * nrm(crs(sub(ld(pos + 3 * i1), a), sub(ld(pos + 3 * i2), a)));
                M[i0] += la / 3.;
                M[i1] += la / 3.;
                M[i2] += la / 3.;
            }
            for (int64_t i = 0; i < nv; ++i)
                for (int k = 0; k < 3; ++k) {
                    vel[3 * i + k] += F[3 * i + k] / M[i] - damping * vel[3 * i + k];
                    pos[3 * i + k] += vel[3 * i + k];
                }
            double st[5];
            orc_particle_update(nv, pos, nt, tri, st);
            orc_membrane_forces(ORC_MODEL_RBC_WLCPOW, prm, nv, rest, nt, tri, tri_area, A0, nl, links, link_len, np,
                                pairs, pair_cs, pos, st[0], st[1], F);
            if (st[0] != st[0]) {
                damping *= 2.;
                success = 0;
                break;
            }
            if (it == 2 * n_it) break;
        }
        if (success) break;
    }
    if (vel_out) memcpy(vel_out, vel, sizeof(double) * 3 * nv);
    free(F0);
    free(F);
    free(vel);
    free(M);
    return damping;
}
