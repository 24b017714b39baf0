// Random initial placement of the reference's particle drivers, host side (no device code):
// ParticlePositionInitializer (src/fsi/ParticlePositionInitializer.hh:17-80) and the random
// orientations of progs/common/create_particles.h:80-93, drawn from the same pseudo-random
// sequence as the C library's rand() on glibc, so that a seed gives the reference's positions
// and orientations bit for bit.
#include "bib_internal.h"

#include <cmath>
#include <limits>

namespace {

// glibc's rand() / random() (the default TYPE_3 state): an additive lagged Fibonacci
// generator x_i = x_{i-3} + x_{i-31} (mod 2^32) returning x_i >> 1, seeded by srand(seed)
// through the Lehmer generator x_i = 16807 x_{i-1} mod (2^31 - 1) for x_1 .. x_30, with the
// first 310 outputs discarded.  RAND_MAX = 2^31 - 1.
class GlibcRand {
public:
    explicit GlibcRand(uint32_t seed) {
        int32_t s = (int32_t)(seed == 0 ? 1 : seed);
        r_[0] = (uint32_t)s;
        for (int i = 1; i < 31; ++i) {
            int64_t v = (16807LL * (int64_t)(int32_t)r_[i - 1]) % 2147483647LL;
            if (v < 0) v += 2147483647LL;
            r_[i] = (uint32_t)v;
        }
        for (int i = 31; i < 34; ++i) r_[i] = r_[i - 31];
        n_ = 34;
        for (int i = 34; i < 344; ++i) step();
    }
    uint32_t next() { return step() >> 1; }

private:
    uint32_t step() {
        // ring of the last 34 values; index n_ is the next one
        const uint32_t v = r_[(n_ - 31) % 34] + r_[(n_ - 3) % 34];
        r_[n_ % 34] = v;
        ++n_;
        return v;
    }
    uint32_t r_[34];
    uint64_t n_;
};

constexpr double kRandMax = 2147483647.0;

}  // namespace

extern "C" {

bib_status bib_initial_distribution(const int64_t* box, const double* pipe, int32_t ntypes, const int64_t* counts,
                                    const double* radii, double max_radius, uint32_t seed, int64_t max_tries,
                                    double* pos, double* quat) {
    if (!box || ntypes < 1 || !counts || !radii || !pos || !quat || !(max_radius > 0) || max_tries < 1)
        return BIB_EINVAL;
    int64_t total = 0;
    for (int t = 0; t < ntypes; ++t) {
        if (counts[t] < 0 || !(radii[t] > 0) || 2 * radii[t] > 2 * max_radius) return BIB_EINVAL;
        total += counts[t];
    }
    GlibcRand rng(seed);
    auto uniform = [&rng]() { return (double)rng.next() / kRandMax; };
    // ParticlePositionInitializer::generate_points per type, in type order: a uniform position in
    // the box shrunk by the radius, inside the boundary by the radius, not overlapping any earlier
    // particle (the initializer's grid of cells >= 2 max_radius finds every such pair)
    std::vector<double> radius(total);
    int64_t n = 0;
    for (int t = 0; t < ntypes; ++t) {
        const double r = radii[t];
        for (int64_t it = 0; it < counts[t]; ++it) {
            bool ok = false;
            double p[3];
            for (int64_t tries = 0; tries < max_tries && !ok; ++tries) {
                for (int a = 0; a < 3; ++a)
                    p[a] = (double)box[2 * a] + r + uniform() * ((double)(box[2 * a + 1] - box[2 * a]) - 2 * r);
                ok = true;
                if (pipe) {  // PipeBoundary::contains(pos, margin = r)
                    const double dy = p[1] - pipe[0], dz = p[2] - pipe[1];
                    ok = (dy * dy + dz * dz) < (pipe[2] - r) * (pipe[2] - r);
                }
                for (int64_t j = 0; ok && j < n; ++j) {
                    const double dx = pos[3 * j] - p[0], dy = pos[3 * j + 1] - p[1], dz = pos[3 * j + 2] - p[2];
                    if (dx * dx + dy * dy + dz * dz < (radius[j] + r) * (radius[j] + r)) ok = false;
                }
            }
            if (!ok) return BIB_EOVERFLOW;  // no free position within max_tries draws
            for (int a = 0; a < 3; ++a) pos[3 * n + a] = p[a];
            radius[n] = r;
            ++n;
        }
    }
    // random orientations (create_particles.h:80-93): an axis of three uniforms drawn last to
    // first (the order g++ evaluates the three arguments of the reference's Array constructor),
    // then an angle; a zero-length axis gives the identity and draws no angle
    for (int64_t i = 0; i < total; ++i) {
        double d[3];
        d[2] = uniform();
        d[1] = uniform();
        d[0] = uniform();
        const double dn = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        double* q = quat + 4 * i;
        if (dn > std::numeric_limits<double>::epsilon()) {
            const double theta = 2. * M_PI * (double)rng.next() / kRandMax;  // (2 pi r) / RAND_MAX
            const double s = std::sin(theta / 2);
            q[0] = std::cos(theta / 2);
            q[1] = s * (d[0] / dn);
            q[2] = s * (d[1] / dn);
            q[3] = s * (d[2] / dn);
        } else {
            q[0] = 1.0;
            q[1] = q[2] = q[3] = 0.0;
        }
    }
    return BIB_OK;
}

}  // extern "C"
