// Oracle harness: runs the REFERENCE's own FP64 code (Palabos + src/fsi of
// niclasberg/biblbm, compiled in place from the reference sources) on inputs
// written by tests/golden/make_golden.py and dumps what it computes.
//
// Test infrastructure only.  Nothing here is linked into the product.
//
// Cases (argv[1]):
//   lbm     collide-and-stream on a periodic box or in simple shear with the
//           finite-difference velocity walls of progs/common/shear_flow_setup.h:51-96
//   ibm     coupled IB-LBM steps in the order of
//           progs/capsule_in_shear/capsule_in_shear.cpp:187-227
//   forces  one call of a particle's compute_forces() at given vertex positions
//   interp  Roma / Peskin interpolation and spreading through the fsi templates
//           (ImmersedBoundaryDynamics_interpolation.hh, ImmersedBoundaryDynamics_forces.hh)
//   shape   ParticleShape rest geometry and connectivity (ParticleShape.hh:21-212)
//   inertia DeformableParticle3D::compute_moment_of_intertia (DeformableParticle3D.hh:173-272)
//   pipe    body-force flow in a pipe along x with the first-order walls of
//           progs/rbc_in_pipe/rbc_in_pipe.cpp:306-318 (BounceBack outside PipeBoundary,
//           NoDynamics beyond radius + 1), in a periodic box
//   pipe_guo the same flow with the second-order walls: GuoRigidWallBoundary on the pipe
//           (rbc_in_pipe.cpp:303-305, fsi/GuoBoundaryCondition.hh) and NoDynamics beyond radius + 1
//   ibm_pipe coupled IB-LBM steps of a capsule near the wall of a pipe with second-order walls:
//           ImmersedBoundaryDynamics3D::set_boundary, i.e. the TopHat near-wall blend of the
//           interpolation and spreading (_interpolation.hh:181-230, _forces.hh:192-237) and the
//           ray-traced wall reflection of the move (DeformableParticle3D.hh:26-51)
//   reflect  DeformableParticle3D::move_vertices(boundary) of given positions and velocities
//   interact the vertex forces of one IB step with a particle-particle interaction
//           (add_pp_force, CollisionForces.h) and a wall interaction decorator
//           (add_force_decorator, ForceDecorator.hh) on parallel plates (Boundary.h:305-365)
//   plb     the particle output formats of particles with given positions, velocities and
//           forces: save_checkpoint (ImmersedBoundaryDynamics_io.hh:17-73),
//           write_particles_as_vtk (_io.hh:161-176, ParticleBase.hh:270-390) and
//           write_lightweight_particle_data (_io.hh:178-199, DeformableParticle3D.hh:318-333),
//           written under out/ of the working directory, plus the registered particle type ids
//   lattice_save  parallelIO::save(lattice, name, false) (io/multiBlockWriter3D.cpp:53-137, 201-213)
//           of a lattice with given populations, forces and phase: out/ckpt.plb + out/ckpt.dat
//           for the default one-block lattice, out/blocks.plb + .dat for the same data on a
//           lattice of bx x by x bz blocks
//   calibrate  the RBC shape calibration of progs/common/calibrate_rbc_shape.h: create_rbc_params
//           (:72-110) on a shape, shrink_rbc_volume (:12-69) to a volume fraction, then
//           set_minor_axis_orientation onto z (DeformableParticle3D.hh:85-144) as
//           RBCShapeInitializer::shrink_volume (:180-185) does
//   initial  the random placement of progs/common/create_particles.h:37-93: srand(seed), then
//           ParticlePositionInitializer::generate_points per particle type inside a PipeBoundary
//           and one random orientation quaternion per particle, drawn as the driver draws them
//   lattice_load  parallelIO::load(name, lattice, false) (io/multiBlockReader3D.cpp:135-268) of
//           in/ckpt.plb into a fresh lattice; dumps its populations, forces and phase
//   coprocessor  D3Q19ExampleCoProcessor3D (coProcessors/coProcessor3D.hh:34-78): addDomain,
//           send of given bytes, collideAndStream, receive
//   create  the reference's own create_particles (progs/common/create_particles.h) for capsule
//           templates of given shapes in a pipe along x: random placement at 20 % scale, growth of
//           rigid copies over its 40000 iterations, deformable particles placed at the result
//   grow    the growth loop of create_particles (:127-161) from given centres and orientations,
//           with a given iteration count, dumping centres, orientations, vertex positions and
//           vertex forces after chosen iterations
//
// Array conventions: lattice fields are (components, nz, ny, nx) with x fastest.
#define FSI_PROFILE
#include "palabos3D.h"
#include "palabos3D.hh"
#include "fsi/headers.h"
#include "fsi/headers.hh"
#include "fsi/GuoBoundaryCondition.h"
#include "fsi/GuoBoundaryCondition.hh"
#include "calibrate_rbc_shape.h"
#include "fsi/ParticlePositionInitializer.h"
#include "fsi/ParticlePositionInitializer.hh"

#include <string>
#include <vector>
#include <sys/stat.h>
#include "rec_io.h"

using namespace plb;
using namespace fsi;
using recio::Bundle;
using recio::shp;

#define DESCRIPTOR descriptors::ForcedPhaseD3Q19Descriptor
typedef double T;
typedef MultiBlockLattice3D<T, DESCRIPTOR> Lattice;

// The globals progs/common/create_particles.h reads, declared as its driver declares them
// (progs/rbc_in_pipe_distribution/rbc_in_pipe.cpp:19, 31, 39, 47-52).
typedef Periodicity3D<double, true, false, false> Periodicity;
struct ParticleTmp {
    ParticleBase3D<double>* particle;
    std::string name;
    double numParticles;
};
std::vector<ParticleTmp> particleTypes;
PipeBoundary<double> pipe_boundary;
bool load_checkpoint = false;
#include "create_particles.h"

static const int Q = 19;

// ---------------------------------------------------------------------------
// shear flow setup, same steps as progs/common/shear_flow_setup.h:51-96
static T shear_velocity(plint iY, plint Ny, T U) {
    const T b = Ny - 1;
    const T y = 2.0 * (T)iY / b - 1;
    return U * y;
}
struct ShearRhoU {
    plint ny; T U;
    ShearRhoU(plint ny_, T U_) : ny(ny_), U(U_) {}
    void operator()(plint, plint iY, plint, T& rho, Array<T, 3>& u) const {
        rho = (T)1; u[0] = shear_velocity(iY, ny, U); u[1] = T(); u[2] = T();
    }
};
struct ShearU {
    plint ny; T U;
    ShearU(plint ny_, T U_) : ny(ny_), U(U_) {}
    void operator()(plint, plint iY, plint, Array<T, 3>& u) const {
        u[0] = shear_velocity(iY, ny, U); u[1] = T(); u[2] = T();
    }
};
static void shear_setup(Lattice& lattice, T U, OnLatticeBoundaryCondition3D<T, DESCRIPTOR>& bc) {
    const plint nx = lattice.getNx(), ny = lattice.getNy(), nz = lattice.getNz();
    Box3D top(0, nx - 1, ny - 1, ny - 1, 0, nz - 1);
    Box3D bottom(0, nx - 1, 0, 0, 0, nz - 1);
    lattice.periodicity().toggle(0, true);
    lattice.periodicity().toggle(2, true);
    bc.addVelocityBoundary1N(bottom, lattice);
    bc.addVelocityBoundary1P(top, lattice);
    initializeAtEquilibrium(lattice, lattice.getBoundingBox(), ShearRhoU(ny, U));
    setBoundaryVelocity(lattice, lattice.getBoundingBox(), ShearU(ny, U));
    lattice.initialize();
}

// ---------------------------------------------------------------------------
static size_t lidx(plint x, plint y, plint z, plint nx, plint ny) { return (size_t)x + nx * ((size_t)y + ny * (size_t)z); }

// With PLB_MPI_PARALLEL, MultiBlockLattice3D::get() returns a proxy cell whose
// population writes do not reach the blocks
// (parallelism/parallelMultiBlockLattice3D.hh:69-87), so cells are reached
// through the single atomic block (fsi requires exactly one block per rank,
// ImmersedBoundaryDynamics.hh:51-54).
static plb::Cell<T, DESCRIPTOR>& cell_at(Lattice& lat, plint x, plint y, plint z) {
    plint id = lat.getLocalInfo().getBlocks()[0];
    SmartBulk3D bulk(lat.getMultiBlockManagement(), id);
    return lat.getComponent(id).get(bulk.toLocalX(x), bulk.toLocalY(y), bulk.toLocalZ(z));
}
static Array<T, 3>& vel_at(MultiTensorField3D<T, 3>& f, plint x, plint y, plint z) {
    plint id = f.getLocalInfo().getBlocks()[0];
    SmartBulk3D bulk(f.getMultiBlockManagement(), id);
    return f.getComponent(id).get(bulk.toLocalX(x), bulk.toLocalY(y), bulk.toLocalZ(z));
}

static void dump_lattice(recio::Writer& w, const std::string& tag, Lattice& lattice) {
    const plint nx = lattice.getNx(), ny = lattice.getNy(), nz = lattice.getNz();
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> f(Q * n), F(3 * n);
    for (plint z = 0; z < nz; ++z)
        for (plint y = 0; y < ny; ++y)
            for (plint x = 0; x < nx; ++x) {
                plb::Cell<T, DESCRIPTOR>& c = cell_at(lattice, x, y, z);
                size_t k = lidx(x, y, z, nx, ny);
                for (int i = 0; i < Q; ++i) f[i * n + k] = c[i];
                for (int d = 0; d < 3; ++d) F[d * n + k] = c.getExternal(0)[d];
            }
    w.d("fbar_" + tag, shp(Q, nz, ny, nx), f);
    w.d("force_" + tag, shp(3, nz, ny, nx), F);
}

static void dump_velocity(recio::Writer& w, const std::string& tag, Lattice& lattice) {
    const plint nx = lattice.getNx(), ny = lattice.getNy(), nz = lattice.getNz();
    const size_t n = (size_t)nx * ny * nz;
    std::auto_ptr<MultiTensorField3D<T, 3> > vel = generateMultiTensorField<T, 3>(lattice.getBoundingBox());
    computeVelocity(lattice, *vel, lattice.getBoundingBox());
    std::vector<double> u(3 * n);
    for (plint z = 0; z < nz; ++z)
        for (plint y = 0; y < ny; ++y)
            for (plint x = 0; x < nx; ++x) {
                Array<T, 3>& v = vel_at(*vel, x, y, z);
                size_t k = lidx(x, y, z, nx, ny);
                for (int d = 0; d < 3; ++d) u[d * n + k] = v[d];
            }
    w.d("u_" + tag, shp(3, nz, ny, nx), u);
}

// the phase external (the voxelization's output), ImmersedBoundaryDynamics_voxelization.hh:106-115
static void dump_phase(recio::Writer& w, const std::string& tag, Lattice& lattice) {
    const plint nx = lattice.getNx(), ny = lattice.getNy(), nz = lattice.getNz();
    std::vector<double> ph((size_t)nx * ny * nz);
    for (plint z = 0; z < nz; ++z)
        for (plint y = 0; y < ny; ++y)
            for (plint x = 0; x < nx; ++x) ph[lidx(x, y, z, nx, ny)] = cell_at(lattice, x, y, z).getExternal(0)[3];
    w.d("phase_" + tag, shp(nz, ny, nx), ph);
}

static void load_lattice(const Bundle& in, Lattice& lattice, bool pops) {
    const plint nx = lattice.getNx(), ny = lattice.getNy(), nz = lattice.getNz();
    const size_t n = (size_t)nx * ny * nz;
    const recio::Array* f = pops ? &recio::need(in, "fbar") : 0;
    const recio::Array* F = recio::has(in, "force") ? &recio::need(in, "force") : 0;
    const recio::Array* ph = recio::has(in, "phase") ? &recio::need(in, "phase") : 0;
    for (plint z = 0; z < nz; ++z)
        for (plint y = 0; y < ny; ++y)
            for (plint x = 0; x < nx; ++x) {
                plb::Cell<T, DESCRIPTOR>& c = cell_at(lattice, x, y, z);
                size_t k = lidx(x, y, z, nx, ny);
                if (f) for (int i = 0; i < Q; ++i) c[i] = f->d[i * n + k];
                if (F) for (int d = 0; d < 3; ++d) c.getExternal(0)[d] = F->d[d * n + k];
                if (ph) c.getExternal(0)[3] = ph->d[k];
            }
    lattice.duplicateOverlaps(modif::staticVariables);
}

static int run_lbm(const Bundle& in, const char* out) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    const T omega = recio::need(in, "omega").d[0], omega_in = recio::need(in, "omega").d[1];
    const long long walls = recio::inum(in, "walls");
    const long long steps = recio::inum(in, "steps");
    Lattice lattice(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(omega, omega_in));
    lattice.toggleInternalStatistics(false);
    std::auto_ptr<OnLatticeBoundaryCondition3D<T, DESCRIPTOR> > bc(createInterpBoundaryCondition3D<T, DESCRIPTOR>());
    if (recio::has(in, "celltype")) {
        // per-cell dynamics as a driver sets them with defineDynamics (rbc_in_pipe.cpp:307-310):
        // 1 BounceBack, 2 NoDynamics
        const recio::Array& ct = recio::need(in, "celltype");
        for (plint z = 0; z < nz; ++z)
            for (plint y = 0; y < ny; ++y)
                for (plint x = 0; x < nx; ++x) {
                    const long long t = ct.i[lidx(x, y, z, nx, ny)];
                    if (t == 1) defineDynamics(lattice, Box3D(x, x, y, y, z, z), new BounceBack<T, DESCRIPTOR>());
                    else if (t == 2) defineDynamics(lattice, Box3D(x, x, y, y, z, z), new NoDynamics<T, DESCRIPTOR>());
                }
    }
    if (walls == 0) {
        lattice.periodicity().toggleAll(true);
        lattice.initialize();  // sets up the periodic envelope exchange before the state is loaded
        load_lattice(in, lattice, true);
    } else {
        shear_setup(lattice, recio::num(in, "U"), *bc);
        load_lattice(in, lattice, false);
    }
    recio::Writer w(out);
    dump_lattice(w, "0", lattice);
    dump_velocity(w, "0", lattice);
    for (long long it = 0; it < steps; ++it) {
        lattice.collideAndStream();
        if (it == 0) {
            dump_lattice(w, "1", lattice);
            dump_velocity(w, "1", lattice);
        }
    }
    dump_lattice(w, "end", lattice);
    dump_velocity(w, "end", lattice);
    return 0;
}

// Cells outside the pipe get BounceBack; cells outside the pipe widened by (plint)sqrt(2) = 1
// get NoDynamics, the two defineDynamics calls of rbc_in_pipe.cpp:306-318 (domain functionals
// BoundarySurface and BoundaryOutside evaluated on PipeBoundary::contains).
static int run_pipe(const Bundle& in, const char* out) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    const std::vector<double> g = recio::need(in, "pipe").d;  // y0, z0, radius
    const T omega = recio::num(in, "omega");
    const long long steps = recio::inum(in, "steps");
    const std::vector<double> body = recio::need(in, "body").d;
    PipeBoundary<T> pipe(g[0], g[1], g[2], (T)(nx - 1));
    Lattice lattice(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(omega, omega));
    lattice.toggleInternalStatistics(false);
    lattice.periodicity().toggleAll(true);
    std::vector<long long> mask((size_t)nx * ny * nz, 0);
    const plint margin = (plint)std::sqrt(2.0);
    for (plint z = 0; z < nz; ++z)
        for (plint y = 0; y < ny; ++y)
            for (plint x = 0; x < nx; ++x) {
                const Array<T, 3> p((T)x, (T)y, (T)z);
                if (!pipe.contains(p)) mask[lidx(x, y, z, nx, ny)] = 1;
                if (!pipe.contains(p, (T)-margin)) mask[lidx(x, y, z, nx, ny)] = 2;
            }
    for (plint z = 0; z < nz; ++z)
        for (plint y = 0; y < ny; ++y)
            for (plint x = 0; x < nx; ++x) {
                const long long t = mask[lidx(x, y, z, nx, ny)];
                if (t == 1) defineDynamics(lattice, Box3D(x, x, y, y, z, z), new BounceBack<T, DESCRIPTOR>());
                else if (t == 2) defineDynamics(lattice, Box3D(x, x, y, y, z, z), new NoDynamics<T, DESCRIPTOR>());
            }
    const Box3D domain = lattice.getBoundingBox();
    setExternalVector(lattice, domain, DESCRIPTOR<T>::ExternalField::forceBeginsAt, Array<T, 3>(body[0], body[1], body[2]));
    initializeAtEquilibrium(lattice, domain, (T)1, Array<T, 3>(0., 0., 0.));
    lattice.initialize();
    for (long long it = 0; it < steps; ++it) lattice.collideAndStream();
    recio::Writer w(out);
    w.i("mask", shp(nz, ny, nx), mask);
    dump_lattice(w, "end", lattice);
    dump_velocity(w, "end", lattice);
    return 0;
}

static int run_pipe_guo(const Bundle& in, const char* out) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    const std::vector<double> g = recio::need(in, "pipe").d;  // y0, z0, radius
    const T omega = recio::num(in, "omega");
    const long long steps = recio::inum(in, "steps");
    const std::vector<double> body = recio::need(in, "body").d;
    PipeBoundary<T> pipe(g[0], g[1], g[2], (T)(nx - 1));
    Lattice lattice(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(omega, omega));
    lattice.toggleInternalStatistics(false);
    lattice.periodicity().toggleAll(true);
    GuoRigidWallBoundary<T, DESCRIPTOR> walls(pipe, lattice);
    walls.insert();
    const plint margin = (plint)std::sqrt(2.0);
    for (plint z = 0; z < nz; ++z)
        for (plint y = 0; y < ny; ++y)
            for (plint x = 0; x < nx; ++x)
                if (!pipe.contains(Array<T, 3>((T)x, (T)y, (T)z), (T)-margin))
                    defineDynamics(lattice, Box3D(x, x, y, y, z, z), new NoDynamics<T, DESCRIPTOR>());
    const Box3D domain = lattice.getBoundingBox();
    setExternalVector(lattice, domain, DESCRIPTOR<T>::ExternalField::forceBeginsAt, Array<T, 3>(body[0], body[1], body[2]));
    initializeAtEquilibrium(lattice, domain, (T)1, Array<T, 3>(0., 0., 0.));
    lattice.initialize();
    recio::Writer w(out);
    dump_lattice(w, "0", lattice);
    std::vector<long long> loc, dir;
    std::vector<double> delta;
    for (GuoRigidWallBoundary<T, DESCRIPTOR>::iterator it = walls.begin(); it != walls.end(); ++it) {
        loc.push_back(it->location.x), loc.push_back(it->location.y), loc.push_back(it->location.z);
        dir.push_back(it->direction.x), dir.push_back(it->direction.y), dir.push_back(it->direction.z);
        delta.push_back(it->delta);
    }
    const long long nw = (long long)delta.size();
    w.i("wall_loc", shp(nw, 3), loc);
    w.i("wall_dir", shp(nw, 3), dir);
    w.d("wall_delta", shp(nw), delta);
    for (long long it = 0; it < steps; ++it) {
        lattice.collideAndStream();
        if (it == 0) dump_lattice(w, "1", lattice);
    }
    dump_lattice(w, "end", lattice);
    dump_velocity(w, "end", lattice);
    return 0;
}

// ---------------------------------------------------------------------------
// Particles

// Composite membrane used by the benchmark's RBC configurations: the capsule's
// Skalak in-plane law (DeformableCapsule.hh:68-150) plus the RBC model's global /
// local area, volume and dihedral-bending terms (RBCParticle.hh:175-246).  The RBC
// part is evaluated by a genuine RBCParticle with zero shear modulus, whose WLC-POW
// link term is then identically zero (ks = kp = 0, RBCParticle.hh:27-44).
class SkalakBendingParticle : public DeformableCapsuleParticle<T> {
public:
    SkalakBendingParticle(const ParticleShape<T>* s, const CapsuleParameters<T>& cp, const RBCParameters<T>& rp)
        : DeformableCapsuleParticle<T>(s, cp), rbc_(s, rp) {}
    virtual SkalakBendingParticle* clone() const { return new SkalakBendingParticle(*this); }
    virtual void compute_forces() {
        DeformableCapsuleParticle<T>::compute_forces();
        for (plint i = 0; i < this->count_nodes(); ++i) rbc_.get_node(i).pos = this->get_node(i).pos;
        rbc_.update();
        rbc_.reset_forces();
        rbc_.compute_forces();
        for (plint i = 0; i < this->count_nodes(); ++i) this->get_node(i).force += rbc_.get_node(i).force;
    }
private:
    RBCParticle<T> rbc_;
};

// DeformableCapsuleParticle has no setter for its shear law; it is serialised
// (DeformableCapsule.hh:215-221), so select it by pack -> patch -> unpack.
static void select_capsule_law(DeformableCapsuleParticle<T>& p, int skalak) {
    std::vector<char> buf;
    p.pack(buf);
    size_t off = sizeof(plint) + sizeof(pluint) + sizeof(plint) + sizeof(bool) + (size_t)p.count_nodes() * 9 * sizeof(T);
    int law = skalak ? 0 : 1;  // enum ShearModel {Skalak, NeoHookean}
    std::memcpy(&buf[off], &law, sizeof(int));
    char* it = &buf[sizeof(plint) + sizeof(pluint)];
    p.unpack(it);
}

struct ParticleSpec {
    long long model;  // 0 capsule NeoHookean, 1 capsule Skalak, 2 RBC (WLC-POW), 3 Skalak + bending composite
    std::vector<double> prm;
};

static ParticleBase3D<T>* make_particle(const ParticleShape<T>* shape, const ParticleSpec& s) {
    // prm layout: [G, C, nu_s, kb, shear_modulus, L0, k_area_global, k_area_local, k_volume, vol_desired, k_bend, theta0]
    CapsuleParameters<T> cp;
    cp.G = s.prm[0]; cp.C = s.prm[1]; cp.nu_s = s.prm[2]; cp.kb = s.prm[3];
    RBCParameters<T> rp;
    rp.shear_modulus = s.prm[4]; rp.L0 = s.prm[5]; rp.k_area_global = s.prm[6]; rp.k_area_local = s.prm[7];
    rp.k_volume = s.prm[8]; rp.vol_desired = s.prm[9]; rp.k_bend = s.prm[10]; rp.theta0 = s.prm[11];
    if (s.model == 0 || s.model == 1) {
        DeformableCapsuleParticle<T>* p = new DeformableCapsuleParticle<T>(shape, cp);
        select_capsule_law(*p, s.model == 1);
        return p;
    }
    if (s.model == 2) return new RBCParticle<T>(shape, rp);
    SkalakBendingParticle* p = new SkalakBendingParticle(shape, cp, rp);
    select_capsule_law(*p, 1);
    return p;
}

static void store_shape(const Bundle& in, ParticleShapeLibrary<T>& lib, const char* xyz_name) {
    const recio::Array& xyz = recio::need(in, xyz_name);
    const recio::Array& tri = recio::need(in, "tri");
    const unsigned nv = (unsigned)xyz.shape[0], nt = (unsigned)tri.shape[0];
    std::vector<Array<T, 3> > v(nv);
    for (unsigned i = 0; i < nv; ++i) v[i] = Array<T, 3>(xyz.d[3 * i], xyz.d[3 * i + 1], xyz.d[3 * i + 2]);
    std::vector<unsigned> idx(3 * nt);
    for (unsigned i = 0; i < 3 * nt; ++i) idx[i] = (unsigned)tri.i[i];
    lib.store_mesh(&v[0], &idx[0], nv, nt, "shape");
}

static void set_positions(ParticleBase3D<T>& p, const recio::Array& pos) {
    for (plint i = 0; i < p.count_nodes(); ++i)
        p.get_node(i).pos = Array<T, 3>(pos.d[3 * i], pos.d[3 * i + 1], pos.d[3 * i + 2]);
    p.update();
}

static ParticleSpec read_spec(const Bundle& in) {
    ParticleSpec s;
    s.model = recio::inum(in, "model");
    s.prm = recio::need(in, "params").d;
    return s;
}

static int run_forces(const Bundle& in, const char* out) {
    ParticleShapeLibrary<T> lib;
    store_shape(in, lib, "rest");
    const ParticleShape<T>* shape = lib.get_by_tag("shape");
    ParticleBase3D<T>* p = make_particle(shape, read_spec(in));
    set_positions(*p, recio::need(in, "pos"));
    p->reset_forces();
    p->compute_forces();
    const plint nv = p->count_nodes();
    std::vector<double> F(3 * nv);
    for (plint i = 0; i < nv; ++i)
        for (int d = 0; d < 3; ++d) F[3 * i + d] = p->get_node(i).force[d];
    recio::Writer w(out);
    w.d("force", shp(nv, 3), F);
    w.d("area", shp(1), std::vector<double>(1, p->area()));
    w.d("volume", shp(1), std::vector<double>(1, p->volume()));
    std::vector<double> com(3);
    for (int d = 0; d < 3; ++d) com[d] = p->center_of_mass()[d];
    w.d("com", shp(3), com);
    delete p;
    return 0;
}

template <class Periodicity>
static int run_ibm_impl(const Bundle& in, const char* out) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    const T tau = recio::num(in, "tau");
    const T lambda = recio::has(in, "lambda") ? recio::num(in, "lambda") : 1.0;
    const long long walls = recio::inum(in, "walls");
    const long long steps = recio::inum(in, "steps");
    const T tau_inner = 0.5 + lambda * (tau - 0.5);
    const T omega = 1. / tau, omega_inner = 1. / tau_inner;

    ParticleShapeLibrary<T> lib;
    store_shape(in, lib, "rest");
    const ParticleShape<T>* shape = lib.get_by_tag("shape");
    ParticleBase3D<T>* proto = make_particle(shape, read_spec(in));
    set_positions(*proto, recio::need(in, "pos"));

    Lattice lattice(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(omega, omega_inner));
    lattice.toggleInternalStatistics(false);
    Box3D domain = lattice.getBoundingBox();
    std::auto_ptr<OnLatticeBoundaryCondition3D<T, DESCRIPTOR> > bc(createInterpBoundaryCondition3D<T, DESCRIPTOR>());
    if (walls == 1) {
        shear_setup(lattice, recio::num(in, "U"), *bc);
    } else {
        lattice.periodicity().toggleAll(true);
        initializeAtEquilibrium(lattice, domain, (T)1, Array<T, 3>(0., 0., 0.));
        lattice.initialize();
    }
    ImmersedBoundaryDynamics3D<T, DESCRIPTOR, Periodicity> fsi(lattice, lib);
    std::auto_ptr<MultiTensorField3D<T, 3> > velocity = generateMultiTensorField<T, 3>(domain);
    fsi.add_particle(proto);
    fsi.init();
    std::vector<double> phase0;
    {
        const size_t n = (size_t)nx * ny * nz;
        phase0.resize(n);
        for (plint z = 0; z < nz; ++z)
            for (plint y = 0; y < ny; ++y)
                for (plint x = 0; x < nx; ++x) phase0[lidx(x, y, z, nx, ny)] = cell_at(lattice, x, y, z).getExternal(0)[3];
    }

    const plint nv = proto->count_nodes();
    std::vector<double> pos((steps + 1) * nv * 3), vel(steps * nv * 3), frc(steps * nv * 3);
    std::vector<double> vol(steps + 1), area(steps + 1), com((steps + 1) * 3), inertia((steps + 1) * 9);
    std::vector<double> body(3, 0.0);
    if (recio::has(in, "body")) body = recio::need(in, "body").d;

    for (long long it = 0; it <= steps; ++it) {
        ParticleBase3D<T>* p = 0;
        fsi.get_particle(0, p);
        for (plint i = 0; i < nv; ++i)
            for (int d = 0; d < 3; ++d) pos[(it * nv + i) * 3 + d] = p->get_node(i).pos[d];
        vol[it] = p->volume();
        area[it] = p->area();
        for (int d = 0; d < 3; ++d) com[it * 3 + d] = p->center_of_mass()[d];
        Matrix<T, 3> I;
        dynamic_cast<DeformableParticle3D<T>*>(p)->compute_moment_of_intertia(I);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) inertia[it * 9 + a * 3 + b] = I(a, b);
        if (it == steps) break;

        computeVelocity(lattice, *velocity, domain);
        setExternalVector(lattice, domain, DESCRIPTOR<T>::ExternalField::forceBeginsAt, Array<T, 3>(body[0], body[1], body[2]));
        applyProcessingFunctional(wrap_ibm_dynamics3D(fsi), domain, lattice, *velocity);
        fsi.get_particle(0, p);
        for (plint i = 0; i < nv; ++i)
            for (int d = 0; d < 3; ++d) {
                vel[(it * nv + i) * 3 + d] = p->get_node(i).vel[d];
                frc[(it * nv + i) * 3 + d] = p->get_node(i).force[d];
            }
        if (it == 0) {
            recio::Writer w0((std::string(out) + ".step0").c_str());
            dump_lattice(w0, "spread", lattice);
        }
        lattice.collideAndStream();
    }
    recio::Writer w(out);
    w.d("pos", shp(steps + 1, nv, 3), pos);
    w.d("vel", shp(steps, nv, 3), vel);
    w.d("force", shp(steps, nv, 3), frc);
    w.d("volume", shp(steps + 1), vol);
    w.d("area", shp(steps + 1), area);
    w.d("com", shp(steps + 1, 3), com);
    w.d("inertia", shp(steps + 1, 3, 3), inertia);
    dump_lattice(w, "end", lattice);
    dump_velocity(w, "end", lattice);
    w.d("phase_0", shp(nz, ny, nx), phase0);
    dump_phase(w, "end", lattice);
    delete proto;
    return 0;
}

static int run_ibm(const Bundle& in, const char* out) {
    if (recio::inum(in, "walls") == 1) return run_ibm_impl<Periodicity3D<T, true, false, true> >(in, out);
    return run_ibm_impl<Periodicity3D<T, true, true, true> >(in, out);
}

// ---------------------------------------------------------------------------
// Interpolation / spreading through the fsi templates with either kernel.
template <class Periodicity, class Dirac>
static int run_interp_impl(const Bundle& in, const char* out) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    const size_t n = (size_t)nx * ny * nz;
    Box3D dom(0, nx - 1, 0, ny - 1, 0, nz - 1);
    typename Periodicity::ArithmeticType arith = Periodicity::create_arithmetic(dom);

    TensorField3D<T, 3> velocity(nx, ny, nz);
    const recio::Array& u = recio::need(in, "u");
    for (plint z = 0; z < nz; ++z)
        for (plint y = 0; y < ny; ++y)
            for (plint x = 0; x < nx; ++x)
                for (int d = 0; d < 3; ++d) velocity.get(x, y, z)[d] = u.d[d * n + lidx(x, y, z, nx, ny)];

    const recio::Array& pos = recio::need(in, "pos");
    const recio::Array& frc = recio::need(in, "nforce");
    const plint nn = pos.shape[0];
    std::vector<NonLocalNode<T> > nodes(nn);
    for (plint i = 0; i < nn; ++i) {
        nodes[i].pos = Array<T, 3>(pos.d[3 * i], pos.d[3 * i + 1], pos.d[3 * i + 2]);
        nodes[i].force = Array<T, 3>(frc.d[3 * i], frc.d[3 * i + 1], frc.d[3 * i + 2]);
        nodes[i].vel.resetToZero();
    }
    recio::Writer w(out);
    std::vector<double> v(3 * nn);

    interpolation::interpolate<T, typename Periodicity::ArithmeticType, NonLocalNode<T>, Dirac>(dom, velocity, nodes, arith);
    for (plint i = 0; i < nn; ++i)
        for (int d = 0; d < 3; ++d) v[3 * i + d] = nodes[i].vel[d];
    w.d("vel_general", shp(nn, 3), v);

    // The bulk fast paths skip all range checks: only nodes whose support box lies
    // inside the field are valid for them (the IB class guarantees that through
    // its bulk_domain, ImmersedBoundaryDynamics.hh:63-65).
    std::vector<NonLocalNode<T> > bulk_nodes;
    std::vector<long long> bulk_ids;
    for (plint i = 0; i < nn; ++i) {
        Box3D b;
        get_dirac_compact_support_box<T, Dirac>(nodes[i].pos, b);
        if (b.x0 >= 0 && b.x1 <= nx - 1 && b.y0 >= 0 && b.y1 <= ny - 1 && b.z0 >= 0 && b.z1 <= nz - 1) {
            bulk_nodes.push_back(nodes[i]);
            bulk_ids.push_back(i);
        }
    }
    interpolation::interpolate_bulk<T, typename Periodicity::ArithmeticType, NonLocalNode<T>, Dirac>(dom, velocity, bulk_nodes, arith);
    std::vector<double> vb(3 * bulk_nodes.size());
    for (size_t i = 0; i < bulk_nodes.size(); ++i)
        for (int d = 0; d < 3; ++d) vb[3 * i + d] = bulk_nodes[i].vel[d];
    w.d("vel_bulk", shp((long long)bulk_nodes.size(), 3), vb);
    w.i("bulk_ids", shp((long long)bulk_ids.size()), bulk_ids);

    for (int mode = 0; mode < 2; ++mode) {
        BlockLattice3D<T, DESCRIPTOR> lat(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(1., 1.));
        for (plint z = 0; z < nz; ++z)
            for (plint y = 0; y < ny; ++y)
                for (plint x = 0; x < nx; ++x)
                    for (int d = 0; d < 4; ++d) lat.get(x, y, z).getExternal(0)[d] = 0.;
        if (mode == 0)
            spreading::spread_forces<T, DESCRIPTOR, Dirac, typename Periodicity::ArithmeticType, NonLocalNode<T> >(dom, lat, nodes, arith);
        else
            spreading::spread_forces_bulk<T, DESCRIPTOR, Dirac, typename Periodicity::ArithmeticType, NonLocalNode<T> >(dom, lat, bulk_nodes, arith);
        std::vector<double> F(3 * n);
        for (plint z = 0; z < nz; ++z)
            for (plint y = 0; y < ny; ++y)
                for (plint x = 0; x < nx; ++x)
                    for (int d = 0; d < 3; ++d) F[d * n + lidx(x, y, z, nx, ny)] = lat.get(x, y, z).getExternal(0)[d];
        w.d(mode == 0 ? "spread_general" : "spread_bulk", shp(3, nz, ny, nx), F);
    }
    return 0;
}

template <class Periodicity>
static int run_interp_p(const Bundle& in, const char* out) {
    if (recio::inum(in, "dirac") == 1) return run_interp_impl<Periodicity, PeskinDirac<T, 3> >(in, out);
    return run_interp_impl<Periodicity, RomaDirac<T, 3> >(in, out);
}

static int run_interp(const Bundle& in, const char* out) {
    const recio::Array& per = recio::need(in, "periodic");
    int code = (per.i[0] ? 4 : 0) | (per.i[1] ? 2 : 0) | (per.i[2] ? 1 : 0);
    switch (code) {
        case 7: return run_interp_p<Periodicity3D<T, true, true, true> >(in, out);
        case 5: return run_interp_p<Periodicity3D<T, true, false, true> >(in, out);
        case 4: return run_interp_p<Periodicity3D<T, true, false, false> >(in, out);
        default: std::fprintf(stderr, "unsupported periodicity\n"); return 2;
    }
}

// ---------------------------------------------------------------------------
static int run_shape(const Bundle& in, const char* out) {
    ParticleShapeLibrary<T> lib;
    store_shape(in, lib, "rest");
    const ParticleShape<T>* s = lib.get_by_tag("shape");
    recio::Writer w(out);
    std::vector<long long> links;
    std::vector<double> lengths;
    for (typename ParticleShape<T>::link_const_iterator it = s->links_begin(); it != s->links_end(); ++it) {
        links.push_back(it->i0); links.push_back(it->i1); lengths.push_back(it->length);
    }
    w.i("links", shp((long long)lengths.size(), 2), links);
    w.d("link_length", shp((long long)lengths.size()), lengths);
    std::vector<long long> pairs;
    std::vector<double> cs;
    for (typename ParticleShape<T>::triangle_pair_const_iterator it = s->triangle_pairs_begin(); it != s->triangle_pairs_end(); ++it) {
        pairs.push_back(it->i0); pairs.push_back(it->i1); pairs.push_back(it->i2); pairs.push_back(it->i3);
        cs.push_back(it->cos_theta0); cs.push_back(it->sin_theta0);
    }
    w.i("pairs", shp((long long)cs.size() / 2, 4), pairs);
    w.d("pair_cos_sin", shp((long long)cs.size() / 2, 2), cs);
    std::vector<double> ta;
    for (typename ParticleShape<T>::triangle_const_iterator it = s->triangles_begin(); it != s->triangles_end(); ++it) ta.push_back(it->area);
    w.d("tri_area", shp((long long)ta.size()), ta);
    w.d("area", shp(1), std::vector<double>(1, s->get_area()));
    w.d("volume", shp(1), std::vector<double>(1, s->get_volume()));
    std::vector<double> c(3);
    for (int d = 0; d < 3; ++d) c[d] = s->get_center()[d];
    w.d("center", shp(3), c);
    w.d("radius", shp(1), std::vector<double>(1, s->get_radius()));
    return 0;
}

static int run_inertia(const Bundle& in, const char* out) {
    ParticleShapeLibrary<T> lib;
    store_shape(in, lib, "rest");
    DeformableCapsuleParticle<T> p(lib.get_by_tag("shape"), CapsuleParameters<T>());
    set_positions(p, recio::need(in, "pos"));
    Matrix<T, 3> I;
    p.compute_moment_of_intertia(I);
    std::vector<double> v(9);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) v[a * 3 + b] = I(a, b);
    recio::Writer w(out);
    w.d("inertia", shp(3, 3), v);
    w.d("volume", shp(1), std::vector<double>(1, p.volume()));
    return 0;
}

// Potentials of kind 1 (Morse: r_min, beta, strength) or 2 (spring: min_dist, _, strength),
// Potentials.h
template <class PP, class WP>
static int run_interact_impl(const Bundle& in, const char* out, const PP& ppot, const WP& wpot) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    ParticleShapeLibrary<T> lib;
    store_shape(in, lib, "rest");
    const ParticleShape<T>* shape = lib.get_by_tag("shape");
    const ParticleSpec spec = read_spec(in);
    ParticleBase3D<T>* pa = make_particle(shape, spec);
    ParticleBase3D<T>* pb = make_particle(shape, spec);
    set_positions(*pa, recio::need(in, "pos_a"));
    set_positions(*pb, recio::need(in, "pos_b"));

    Lattice lattice(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(1.0, 1.0));
    lattice.toggleInternalStatistics(false);
    Box3D domain = lattice.getBoundingBox();
    lattice.periodicity().toggleAll(true);
    initializeAtEquilibrium(lattice, domain, (T)1, Array<T, 3>(0., 0., 0.));
    lattice.initialize();
    ImmersedBoundaryDynamics3D<T, DESCRIPTOR, Periodicity3D<T, true, true, true> > fsi(lattice, lib);
    const std::vector<double> wy = recio::need(in, "wall_y").d;
    ParallelPlatesBoundary<T> plates(wy[0], wy[1]);
    // a pipe along x instead of the plates when given (y0, z0, radius), as rbc_in_pipe.cpp:154-163
    std::vector<double> pp_geo = recio::has(in, "pipe") ? recio::need(in, "pipe").d : std::vector<double>(3, 0.0);
    PipeBoundary<T> pipe(pp_geo[0], pp_geo[1], pp_geo[2], (T)nx);
    const Boundary<T>& bnd = recio::has(in, "pipe") ? static_cast<const Boundary<T>&>(pipe)
                                                     : static_cast<const Boundary<T>&>(plates);
    WallInteraction<T, WP> wall(bnd, wpot);
    PPPotentialForce<T, PP> pp(ppot);
    fsi.add_force_decorator(&wall);
    fsi.add_pp_force(&pp);
    std::auto_ptr<MultiTensorField3D<T, 3> > velocity = generateMultiTensorField<T, 3>(domain);
    fsi.add_particle(pa);
    fsi.add_particle(pb);
    fsi.init();
    computeVelocity(lattice, *velocity, domain);
    setExternalVector(lattice, domain, DESCRIPTOR<T>::ExternalField::forceBeginsAt, Array<T, 3>(0., 0., 0.));
    applyProcessingFunctional(wrap_ibm_dynamics3D(fsi), domain, lattice, *velocity);
    recio::Writer w(out);
    const char* names[2] = {"force_a", "force_b"};
    for (plint id = 0; id < 2; ++id) {
        ParticleBase3D<T>* p = 0;
        fsi.get_particle(id, p);
        const plint nv = p->count_nodes();
        std::vector<double> F(3 * nv);
        for (plint i = 0; i < nv; ++i)
            for (int d = 0; d < 3; ++d) F[3 * i + d] = p->get_node(i).force[d];
        w.d(names[id], shp(nv, 3), F);
    }
    delete pa;
    delete pb;
    return 0;
}

static int run_ibm_pipe(const Bundle& in, const char* out) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    const std::vector<double> g = recio::need(in, "pipe").d;  // y0, z0, radius
    const T omega = 1. / recio::num(in, "tau");
    const long long steps = recio::inum(in, "steps");
    const std::vector<double> body = recio::need(in, "body").d;
    PipeBoundary<T> pipe(g[0], g[1], g[2], (T)(nx - 1));
    ParticleShapeLibrary<T> lib;
    store_shape(in, lib, "rest");
    const ParticleShape<T>* shape = lib.get_by_tag("shape");
    ParticleBase3D<T>* proto = make_particle(shape, read_spec(in));
    set_positions(*proto, recio::need(in, "pos"));
    Lattice lattice(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(omega, omega));
    lattice.toggleInternalStatistics(false);
    lattice.periodicity().toggleAll(true);
    GuoRigidWallBoundary<T, DESCRIPTOR> walls(pipe, lattice);
    walls.insert();
    const plint margin = (plint)std::sqrt(2.0);
    for (plint z = 0; z < nz; ++z)
        for (plint y = 0; y < ny; ++y)
            for (plint x = 0; x < nx; ++x)
                if (!pipe.contains(Array<T, 3>((T)x, (T)y, (T)z), (T)-margin))
                    defineDynamics(lattice, Box3D(x, x, y, y, z, z), new NoDynamics<T, DESCRIPTOR>());
    const Box3D domain = lattice.getBoundingBox();
    initializeAtEquilibrium(lattice, domain, (T)1, Array<T, 3>(0., 0., 0.));
    lattice.initialize();
    ImmersedBoundaryDynamics3D<T, DESCRIPTOR, Periodicity3D<T, true, true, true> > fsi(lattice, lib);
    fsi.set_boundary(&pipe);
    std::auto_ptr<MultiTensorField3D<T, 3> > velocity = generateMultiTensorField<T, 3>(domain);
    fsi.add_particle(proto);
    fsi.init();
    const plint nv = proto->count_nodes();
    std::vector<double> pos((steps + 1) * nv * 3), vel(steps * nv * 3), frc(steps * nv * 3);
    for (long long it = 0; it <= steps; ++it) {
        ParticleBase3D<T>* p = 0;
        fsi.get_particle(0, p);
        for (plint i = 0; i < nv; ++i)
            for (int d = 0; d < 3; ++d) pos[(it * nv + i) * 3 + d] = p->get_node(i).pos[d];
        if (it == steps) break;
        computeVelocity(lattice, *velocity, domain);
        setExternalVector(lattice, domain, DESCRIPTOR<T>::ExternalField::forceBeginsAt, Array<T, 3>(body[0], body[1], body[2]));
        applyProcessingFunctional(wrap_ibm_dynamics3D(fsi), domain, lattice, *velocity);
        fsi.get_particle(0, p);
        for (plint i = 0; i < nv; ++i)
            for (int d = 0; d < 3; ++d) {
                vel[(it * nv + i) * 3 + d] = p->get_node(i).vel[d];
                frc[(it * nv + i) * 3 + d] = p->get_node(i).force[d];
            }
        if (it == 0) {
            recio::Writer w0((std::string(out) + ".step0").c_str());
            dump_lattice(w0, "spread", lattice);
        }
        lattice.collideAndStream();
    }
    recio::Writer w(out);
    w.d("pos", shp(steps + 1, nv, 3), pos);
    w.d("vel", shp(steps, nv, 3), vel);
    w.d("force", shp(steps, nv, 3), frc);
    dump_lattice(w, "end", lattice);
    dump_velocity(w, "end", lattice);
    delete proto;
    return 0;
}

static int run_reflect(const Bundle& in, const char* out) {
    const std::vector<double> g = recio::need(in, "pipe").d;
    PipeBoundary<T> pipe(g[0], g[1], g[2], (T)100);
    ParticleShapeLibrary<T> lib;
    store_shape(in, lib, "rest");
    ParticleBase3D<T>* p = make_particle(lib.get_by_tag("shape"), read_spec(in));
    set_positions(*p, recio::need(in, "pos"));
    const recio::Array& v = recio::need(in, "vel");
    const plint nv = p->count_nodes();
    for (plint i = 0; i < nv; ++i) p->get_node(i).vel = Array<T, 3>(v.d[3 * i], v.d[3 * i + 1], v.d[3 * i + 2]);
    dynamic_cast<DeformableParticle3D<T>*>(p)->move_vertices(&pipe);
    std::vector<double> P(3 * nv);
    for (plint i = 0; i < nv; ++i)
        for (int d = 0; d < 3; ++d) P[3 * i + d] = p->get_node(i).pos[d];
    recio::Writer w(out);
    w.d("pos", shp(nv, 3), P);
    delete p;
    return 0;
}

static int run_interact(const Bundle& in, const char* out) {
    const long long ppk = recio::inum(in, "pp_kind"), wk = recio::inum(in, "wall_kind");
    const std::vector<double> a = recio::need(in, "pp_params").d, b = recio::need(in, "wall_params").d;
    const MorsePotential<T> ma(a[0], a[1], a[2]), mb(b[0], b[1], b[2]);
    const SpringPotential<T> sa(a[0], a[2]), sb(b[0], b[2]);
    if (ppk == 1 && wk == 1) return run_interact_impl(in, out, ma, mb);
    if (ppk == 1 && wk == 2) return run_interact_impl(in, out, ma, sb);
    if (ppk == 2 && wk == 1) return run_interact_impl(in, out, sa, mb);
    if (ppk == 2 && wk == 2) return run_interact_impl(in, out, sa, sb);
    std::fprintf(stderr, "unknown potential kinds %lld %lld\n", ppk, wk);
    return 2;
}

static void store_shape_as(const Bundle& in, ParticleShapeLibrary<T>& lib, const char* xyz_name,
                           const char* tri_name, const char* tag) {
    const recio::Array& xyz = recio::need(in, xyz_name);
    const recio::Array& tri = recio::need(in, tri_name);
    const unsigned nv = (unsigned)xyz.shape[0], nt = (unsigned)tri.shape[0];
    std::vector<Array<T, 3> > v(nv);
    for (unsigned i = 0; i < nv; ++i) v[i] = Array<T, 3>(xyz.d[3 * i], xyz.d[3 * i + 1], xyz.d[3 * i + 2]);
    std::vector<unsigned> idx(3 * nt);
    for (unsigned i = 0; i < 3 * nt; ++i) idx[i] = (unsigned)tri.i[i];
    lib.store_mesh(&v[0], &idx[0], nv, nt, tag);
}

static int run_plb(const Bundle& in, const char* out) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    ParticleShapeLibrary<T> lib;
    store_shape_as(in, lib, "rest", "tri", "shape");
    store_shape_as(in, lib, "rest_b", "tri_b", "shape_b");
    const recio::Array& models = recio::need(in, "models");
    const recio::Array& shapes = recio::need(in, "shapes");
    const recio::Array& params = recio::need(in, "params");
    const recio::Array& pos = recio::need(in, "pos");
    const recio::Array& vel = recio::need(in, "vel");
    const recio::Array& frc = recio::need(in, "force");
    const long long iter = recio::inum(in, "iter");
    const size_t np = (size_t)models.shape[0];

    Lattice lattice(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(1.0, 1.0));
    lattice.toggleInternalStatistics(false);
    lattice.periodicity().toggleAll(true);
    initializeAtEquilibrium(lattice, lattice.getBoundingBox(), (T)1, Array<T, 3>(0., 0., 0.));
    lattice.initialize();
    ImmersedBoundaryDynamics3D<T, DESCRIPTOR, Periodicity3D<T, true, true, true> > fsi(lattice, lib);
    size_t off = 0;
    for (size_t k = 0; k < np; ++k) {
        ParticleSpec spec;
        spec.model = models.i[k];
        spec.prm.assign(params.d.begin() + 12 * k, params.d.begin() + 12 * (k + 1));
        const ParticleShapeLibrary<T>& clib = lib;  // the non-const get_by_id does not compile
        ParticleBase3D<T>* proto = make_particle(clib.get_by_id(shapes.i[k]), spec);
        for (plint i = 0; i < proto->count_nodes(); ++i)
            proto->get_node(i).pos = Array<T, 3>(pos.d[off + 3 * i], pos.d[off + 3 * i + 1], pos.d[off + 3 * i + 2]);
        proto->update();
        off += 3 * (size_t)proto->count_nodes();
        fsi.add_particle(proto);
        delete proto;
    }
    off = 0;
    for (size_t k = 0; k < np; ++k) {
        ParticleBase3D<T>* p = 0;
        fsi.get_particle((plint)k, p);
        for (plint i = 0; i < p->count_nodes(); ++i) {
            p->get_node(i).vel = Array<T, 3>(vel.d[off + 3 * i], vel.d[off + 3 * i + 1], vel.d[off + 3 * i + 2]);
            p->get_node(i).force = Array<T, 3>(frc.d[off + 3 * i], frc.d[off + 3 * i + 1], frc.d[off + 3 * i + 2]);
        }
        off += 3 * (size_t)p->count_nodes();
    }
    ::mkdir("out", 0777);
    global::directories().setOutputDir("out/");
    fsi.save_checkpoint(FileName("ckpt"));
    fsi.write_particles_as_vtk((pluint)iter);
    fsi.write_lightweight_particle_data((pluint)iter);
    recio::Writer w(out);
    std::vector<long long> ids;
    const ParticleShapeLibrary<T>& clib = lib;
    DeformableCapsuleParticle<T> capsule(clib.get_by_id(0), CapsuleParameters<T>());
    RBCParticle<T> rbc(clib.get_by_id(0));
    ids.push_back(capsule.get_type_id());
    ids.push_back(rbc.get_type_id());
    w.i("type_ids", shp(2), ids);
    return 0;
}

static int run_lattice_save(const Bundle& in, const char* out) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    const std::vector<long long> nb = recio::need(in, "blocks").i;
    Lattice lattice(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(1.0, 1.0));
    lattice.toggleInternalStatistics(false);
    load_lattice(in, lattice, true);
    ::mkdir("out", 0777);
    global::directories().setOutputDir("out/");
    parallelIO::save(lattice, "ckpt", false);
    // the same data on a lattice of several blocks, all on this rank
    SparseBlockStructure3D blocks = createRegularDistribution3D(nx, ny, nz, nb[0], nb[1], nb[2]);
    ExplicitThreadAttribution* threads = new ExplicitThreadAttribution;
    for (plint b = 0; b < (plint)(nb[0] * nb[1] * nb[2]); ++b) threads->addBlock(b, 0);
    MultiBlockLattice3D<T, DESCRIPTOR> multi(MultiBlockManagement3D(blocks, threads, 1),
                                             defaultMultiBlockPolicy3D().getBlockCommunicator(),
                                             defaultMultiBlockPolicy3D().getCombinedStatistics(),
                                             defaultMultiBlockPolicy3D().getMultiCellAccess<T, DESCRIPTOR>(),
                                             new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(1.0, 1.0));
    multi.toggleInternalStatistics(false);
    copy_generic(lattice, lattice.getBoundingBox(), multi, multi.getBoundingBox(), modif::staticVariables);
    parallelIO::save(multi, "blocks", false);
    recio::Writer w(out);
    w.i("nblocks", shp(1), std::vector<long long>(1, (long long)multi.getMultiBlockManagement().getSparseBlockStructure().getBulks().size()));
    return 0;
}

static int run_lattice_load(const Bundle& in, const char* out) {
    const recio::Array& dims = recio::need(in, "dims");
    const plint nx = dims.i[0], ny = dims.i[1], nz = dims.i[2];
    Lattice lattice(nx, ny, nz, new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(1.0, 1.0));
    lattice.toggleInternalStatistics(false);
    global::directories().setInputDir("in/");
    parallelIO::load("ckpt", lattice, false);
    recio::Writer w(out);
    dump_lattice(w, "loaded", lattice);
    dump_phase(w, "loaded", lattice);
    return 0;
}

static int run_calibrate(const Bundle& in, const char* out) {
    ParticleShapeLibrary<T> lib;
    store_shape(in, lib, "rest");
    const ParticleShapeLibrary<T>& clib = lib;
    const ParticleShape<T>* shape = clib.get_by_id(0);
    const std::vector<double> k = recio::need(in, "moduli").d;  // shear modulus, K_area, K_bend
    RBCParameters<T> prm = create_rbc_params(shape, (T)k[0], (T)k[1], (T)k[2]);
    RBCParticle<T> rbc(shape, prm);
    const T vol_final = recio::num(in, "vol_frac") * shape->get_volume();
    shrink_rbc_volume(rbc, vol_final, (int)recio::inum(in, "n_it"), (T)1, (T)recio::num(in, "damping"));
    const plint nv = rbc.count_nodes();
    std::vector<double> shrunk(3 * nv), aligned(3 * nv);
    for (plint i = 0; i < nv; ++i)
        for (int d = 0; d < 3; ++d) shrunk[3 * i + d] = rbc.get_node(i).pos[d];
    rbc.set_minor_axis_orientation(Array<T, 3>(0, 0, 1));
    rbc.params().vol_desired = rbc.volume();
    for (plint i = 0; i < nv; ++i)
        for (int d = 0; d < 3; ++d) aligned[3 * i + d] = rbc.get_node(i).pos[d];
    const RBCParameters<T>& p = prm;
    double pv[12] = {0, 0, 0, 0, p.shear_modulus, p.L0, p.k_area_global, p.k_area_local, p.k_volume, p.vol_desired,
                     p.k_bend, p.theta0};
    recio::Writer w(out);
    w.d("params", shp(12), std::vector<double>(pv, pv + 12));
    w.d("shrunk", shp(nv, 3), shrunk);
    w.d("aligned", shp(nv, 3), aligned);
    w.d("vol_desired", shp(1), std::vector<double>(1, rbc.params().vol_desired));
    w.d("area", shp(1), std::vector<double>(1, rbc.area()));
    return 0;
}

static int run_initial(const Bundle& in, const char* out) {
    const std::vector<long long> b = recio::need(in, "box").i;
    const std::vector<double> pp = recio::need(in, "pipe").d;  // y0, z0, radius
    const std::vector<long long> counts = recio::need(in, "counts").i;
    const std::vector<double> radii = recio::need(in, "radii").d;
    const T max_radius = recio::num(in, "max_radius");
    std::srand((unsigned)recio::inum(in, "seed"));
    PipeBoundary<T> pipe(pp[0], pp[1], pp[2], (T)(b[1] - b[0]));
    ParticlePositionInitializer<T> init(Box3D(b[0], b[1], b[2], b[3], b[4], b[5]), &pipe, max_radius);
    for (size_t t = 0; t < counts.size(); ++t)
        if (!init.generate_points((pluint)counts[t], radii[t], (char)t)) return 3;
    std::vector<double> pos, quat;
    for (size_t t = 0; t < counts.size(); ++t) {
        std::vector<Array<T, 3> > pts;
        init.get_points((char)t, pts);
        for (size_t i = 0; i < pts.size(); ++i)
            for (int d = 0; d < 3; ++d) pos.push_back(pts[i][d]);
    }
    // one orientation per particle, the axis built from three draws in one constructor call as
    // the driver does, the angle from a fourth draw unless the axis is zero
    const size_t n = pos.size() / 3;
    for (size_t i = 0; i < n; ++i) {
        Array<T, 3> dir((T)std::rand() / RAND_MAX, (T)std::rand() / RAND_MAX, (T)std::rand() / RAND_MAX);
        const T dn = norm(dir);
        Quaternion<T> q;
        if (dn > std::numeric_limits<T>::epsilon()) q = Quaternion<T>(2. * M_PI * (T)std::rand() / RAND_MAX, dir / dn);
        for (int k = 0; k < 4; ++k) quat.push_back(q[k]);
    }
    recio::Writer w(out);
    w.d("pos", shp((long long)n, 3), pos);
    w.d("quat", shp((long long)n, 4), quat);
    return 0;
}

// Palabos' example co-processor (coProcessors/coProcessor3D.hh:34-78): addDomain with the given
// omega, send of the given cell-major bytes (19 f-bar per cell, z fastest), one collideAndStream,
// receive; dumps the received bytes as doubles.
static int run_coprocessor(const Bundle& in, const char* out) {
    const std::vector<long long> dims = recio::need(in, "dims").i;
    const T omega = recio::num(in, "omega");
    const std::vector<double> data = recio::need(in, "data").d;
    const plint nx = dims[0], ny = dims[1], nz = dims[2];
    D3Q19ExampleCoProcessor3D<T> cp;
    int handle = -1;
    if (cp.addDomain(nx, ny, nz, omega, handle) != 1) return 3;
    const Box3D box(0, nx - 1, 0, ny - 1, 0, nz - 1);
    std::vector<char> bytes(data.size() * sizeof(double));
    std::memcpy(&bytes[0], &data[0], bytes.size());
    if (cp.send(handle, box, bytes) != 1) return 3;
    const plint steps = recio::inum(in, "steps");
    for (plint s = 0; s < steps; ++s)
        if (cp.collideAndStream(handle) != 1) return 3;
    std::vector<char> back;
    if (cp.receive(handle, box, back) != 1) return 3;
    std::vector<double> res(back.size() / sizeof(double));
    std::memcpy(&res[0], &back[0], back.size());
    recio::Writer w(out);
    w.d("data", shp(nx, ny, nz, Q), res);
    return 0;
}


// create_particles on a lattice over `box` (x0, x1, y0, y1, z0, z1; periodic in x as the pipe
// drivers), pipe = (y0, z0, radius, length), capsule templates of the shapes rest<t> / tri<t>
// with counts[t] particles each, srand(seed).  Dumps the vertex positions of the particles it
// adds, in id order.
static Lattice* pipe_lattice(const std::vector<long long>& b) {
    Lattice* lattice = generateMultiBlockLattice<T, DESCRIPTOR>(Box3D(b[0], b[1], b[2], b[3], b[4], b[5]),
                                                               new GuoExternalForceVOFDynamics<T, DESCRIPTOR>(1.0, 1.0), 1)
                           .release();
    lattice->periodicity().toggle(0, Periodicity::get_x());
    lattice->periodicity().toggle(1, Periodicity::get_y());
    lattice->periodicity().toggle(2, Periodicity::get_z());
    lattice->toggleInternalStatistics(false);
    return lattice;
}

static void store_typed_shapes(const Bundle& in, ParticleShapeLibrary<T>& lib, long long ntypes) {
    for (long long t = 0; t < ntypes; ++t) {
        char xn[32], tn[32], tag[32];
        std::sprintf(xn, "rest%lld", t);
        std::sprintf(tn, "tri%lld", t);
        std::sprintf(tag, "type%lld", t);
        store_shape_as(in, lib, xn, tn, tag);
    }
}

static int run_create(const Bundle& in, const char* out) {
    const std::vector<long long> b = recio::need(in, "box").i;
    const std::vector<double> pp = recio::need(in, "pipe").d;
    const std::vector<long long> counts = recio::need(in, "counts").i;
    Lattice* lattice = pipe_lattice(b);
    pipe_boundary = PipeBoundary<T>(pp[0], pp[1], pp[2], pp[3]);
    ParticleShapeLibrary<T> lib;
    store_typed_shapes(in, lib, (long long)counts.size());
    particleTypes.clear();
    for (size_t t = 0; t < counts.size(); ++t) {
        char tag[32];
        std::sprintf(tag, "type%d", (int)t);
        ParticleTmp pt;
        pt.particle = new DeformableCapsuleParticle<T>(lib.get_by_tag(tag), CapsuleParameters<T>());
        pt.name = std::string("rigid_") + tag;
        pt.numParticles = (double)counts[t];
        particleTypes.push_back(pt);
    }
    ImmersedBoundaryDynamics3D<T, DESCRIPTOR, Periodicity> fsi(*lattice, lib);
    global::directories().setOutputDir("out/");
    io::mkdir("out/");
    std::srand((unsigned)recio::inum(in, "seed"));
    create_particles<T>(fsi, *lattice);
    std::vector<double> pos;
    plint n = 0;
    for (plint id = 0;; ++id) {
        ParticleBase3D<T>* p = 0;
        if (!fsi.get_particle(id, p)) break;
        for (plint i = 0; i < p->count_nodes(); ++i)
            for (int d = 0; d < 3; ++d) pos.push_back(p->get_node(i).pos[d]);
        ++n;
    }
    recio::Writer w(out);
    w.d("pos", shp((long long)(pos.size() / 3), 3), pos);
    w.d("count", shp(1), std::vector<double>(1, (double)n));
    for (size_t t = 0; t < particleTypes.size(); ++t) delete particleTypes[t].particle;
    particleTypes.clear();
    delete lattice;
    return 0;
}

// The body of create_particles' growth loop (create_particles.h:127-161) on rigid copies of the
// shapes rest<t> / tri<t>: particle k on shape[k] starts at com[k] / quat[k], the wall is
// PipeBoundary(wall[0], wall[1], wall[2], box length), the potential SpringPotential(pot[0],
// pot[1]); growth = (initial_scale, density, damping), n_it the iteration the scale reaches 1.
// After the iterations listed in `dump` (counts of iterations run) the centres, orientations,
// vertex positions and vertex forces are written with the count as suffix.
static int run_grow(const Bundle& in, const char* out) {
    const std::vector<long long> b = recio::need(in, "box").i;
    const std::vector<double> wall = recio::need(in, "wall").d;
    const std::vector<double> pot = recio::need(in, "pot").d;
    const std::vector<double> gr = recio::need(in, "growth").d;
    const std::vector<long long> shape = recio::need(in, "shape").i;
    const std::vector<double> com = recio::need(in, "com").d;
    const std::vector<double> quat = recio::need(in, "quat").d;
    const std::vector<long long> dump = recio::need(in, "dump").i;
    const plint Nit = (plint)recio::inum(in, "n_it");
    const long long ntypes = recio::inum(in, "ntypes");
    Lattice* lattice = pipe_lattice(b);
    ParticleShapeLibrary<T> lib;
    store_typed_shapes(in, lib, ntypes);
    ImmersedBoundaryDynamics3D<T, DESCRIPTOR, Periodicity> fsi2(*lattice, lib);
    PipeBoundary<T> boundary2(wall[0], wall[1], wall[2], (T)(b[1] - b[0]));
    std::vector<RigidParticle3D<T>*> rigid;
    for (long long t = 0; t < ntypes; ++t) {
        char tag[32];
        std::sprintf(tag, "type%lld", t);
        RigidParticle3D<T>* r = new RigidParticle3D<T>(lib.get_by_tag(tag));
        r->scale() = gr[0];
        r->density() = gr[1];
        r->damping() = gr[2];
        r->update();
        rigid.push_back(r);
    }
    for (size_t k = 0; k < shape.size(); ++k) {
        RigidParticle3D<T>* p = rigid[shape[k]];
        p->scale() = gr[0];
        p->set_center_of_mass(Array<T, 3>(com[3 * k], com[3 * k + 1], com[3 * k + 2]));
        p->orientation() = fsi::Quaternion<T>(quat[4 * k], quat[4 * k + 1], quat[4 * k + 2], quat[4 * k + 3]);
        p->update();
        fsi2.add_particle(p);
    }
    fsi2.init();
    SpringPotential<T> potential(pot[0], pot[1]);
    recio::Writer w(out);
    size_t next = 0;
    T scale;
    for (plint it = 0; next < dump.size(); ++it) {
        if ((it % 10) == 0) {
            T fraction = (T)it / (T)Nit;
            scale = gr[0] + (1. - gr[0]) * fraction;
            for (ImmersedBoundaryDynamics3D<T, DESCRIPTOR, Periodicity>::ObjMapIterator iter = fsi2.particles_begin();
                 iter != fsi2.particles_end(); ++iter) {
                RigidParticle3D<T>* p = dynamic_cast<RigidParticle3D<T>*>(iter->second);
                if (p) {
                    p->scale() = scale;
                    p->update();
                }
            }
            fsi2.synchronize_particle_states();
        }
        fsi2.compute_collision_forces(potential, &boundary2);
        fsi2.move_vertices();
        if (it + 1 == dump[next]) {
            std::vector<double> c, q, x, f;
            for (plint id = 0; id < (plint)shape.size(); ++id) {
                ParticleBase3D<T>* pb = 0;
                fsi2.get_particle(id, pb);
                RigidParticle3D<T>* p = dynamic_cast<RigidParticle3D<T>*>(pb);
                for (int d = 0; d < 3; ++d) c.push_back(p->center_of_mass()[d]);
                for (int d = 0; d < 4; ++d) q.push_back(p->orientation()[d]);
                for (plint i = 0; i < p->count_nodes(); ++i)
                    for (int d = 0; d < 3; ++d) {
                        x.push_back(p->get_node(i).pos[d]);
                        f.push_back(p->get_node(i).force[d]);
                    }
            }
            char tc[32], tq[32], tx[32], tf[32];
            std::sprintf(tc, "com_%lld", dump[next]);
            std::sprintf(tq, "quat_%lld", dump[next]);
            std::sprintf(tx, "pos_%lld", dump[next]);
            std::sprintf(tf, "force_%lld", dump[next]);
            w.d(tc, shp((long long)shape.size(), 3), c);
            w.d(tq, shp((long long)shape.size(), 4), q);
            w.d(tx, shp((long long)(x.size() / 3), 3), x);
            w.d(tf, shp((long long)(f.size() / 3), 3), f);
            ++next;
        }
    }
    for (size_t t = 0; t < rigid.size(); ++t) delete rigid[t];
    delete lattice;
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: ref_harness <lbm|ibm|forces|interp|shape|inertia> in.rec out.rec\n");
        return 2;
    }
    plbInit(&argc, &argv);
    Bundle in = recio::read_file(argv[2]);
    std::string c = argv[1];
    if (c == "lbm") return run_lbm(in, argv[3]);
    if (c == "ibm") return run_ibm(in, argv[3]);
    if (c == "forces") return run_forces(in, argv[3]);
    if (c == "interp") return run_interp(in, argv[3]);
    if (c == "shape") return run_shape(in, argv[3]);
    if (c == "inertia") return run_inertia(in, argv[3]);
    if (c == "interact") return run_interact(in, argv[3]);
    if (c == "pipe") return run_pipe(in, argv[3]);
    if (c == "pipe_guo") return run_pipe_guo(in, argv[3]);
    if (c == "ibm_pipe") return run_ibm_pipe(in, argv[3]);
    if (c == "reflect") return run_reflect(in, argv[3]);
    if (c == "plb") return run_plb(in, argv[3]);
    if (c == "lattice_save") return run_lattice_save(in, argv[3]);
    if (c == "lattice_load") return run_lattice_load(in, argv[3]);
    if (c == "calibrate") return run_calibrate(in, argv[3]);
    if (c == "initial") return run_initial(in, argv[3]);
    if (c == "coprocessor") return run_coprocessor(in, argv[3]);
    if (c == "create") return run_create(in, argv[3]);
    if (c == "grow") return run_grow(in, argv[3]);
    std::fprintf(stderr, "unknown case %s\n", argv[1]);
    return 2;
}
