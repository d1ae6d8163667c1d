// host_check.cpp -- gvs_host_check: exercises the C++ host layer's drop-in
// classes (the per-call GravitySolver / Integrator / SphSolver interfaces, with
// host arrays) against the device-resident path on the same inputs.  Prints
// one line per check and exits non-zero on the first mismatch.
//
//   1. BruteForce (FP64_EXACT) accumulates: forces on zeroed a equal the
//      resident gvs_compute_forces result bit for bit, and a second call doubles them.
//   2. LeapfrogKDK::step x 50 with BruteForce equals gvs_kdk_steps(50) bit for bit.
//   3. BarnesHut::compute_accelerations equals the resident BH forces bit for bit.
//   4. SphSolver::compute + step_with_sph x 3 on the Evrard sphere equal the
//      resident gvs_sph_compute / gvs_sph_step sequence bit for bit.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gravis.hpp"

using namespace gravis;

namespace {
int failures = 0;

void report(const char *what, bool ok) {
    std::printf("%s %s\n", ok ? "ok  " : "FAIL", what);
    if (!ok) ++failures;
}

bool same(const std::vector<double> &a, const std::vector<double> &b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (!(a[i] == b[i])) return false;
    return true;
}
}  // namespace

int main() {
    try {
        Context ctx(0);
        PlummerSphere ps;
        ps.n = 2000;
        ps.seed = 5;
        const Particles p0 = ps.generate();
        const double eps = ps.suggested_softening(), dt = ps.suggested_dt();

        // 1. BruteForce accumulate semantics
        {
            Particles p = p0;
            p.clear_accelerations();
            BruteForce bf(ctx, eps);
            bf.compute_accelerations(p);
            Particles r = p0;
            upload(ctx, r, false);
            ctx.check(gvs_compute_forces(ctx.get(), GVS_ALGO_DIRECT, GVS_PREC_FP64_EXACT, eps, 0.5));
            download(ctx, r);
            report("BruteForce::compute_accelerations == resident forces", same(p.ax, r.ax) && same(p.az, r.az));
            std::vector<double> twice = p.ax;
            for (double &v : twice) v *= 2.0;
            bf.compute_accelerations(p);
            report("BruteForce accumulates into the caller's arrays", same(p.ax, twice));
        }
        // 2. LeapfrogKDK::step vs resident steps
        {
            Particles p = p0;
            p.clear_accelerations();
            BruteForce bf(ctx, eps);
            bf.compute_accelerations(p);
            LeapfrogKDK kdk(ctx);
            for (int s = 0; s < 50; ++s) kdk.step(p, bf, dt);
            Particles r = p0;
            upload(ctx, r, false);
            ctx.check(gvs_compute_forces(ctx.get(), GVS_ALGO_DIRECT, GVS_PREC_FP64_EXACT, eps, 0.5));
            ctx.check(gvs_kdk_steps(ctx.get(), GVS_ALGO_DIRECT, GVS_PREC_FP64_EXACT, eps, 0.5, dt, 50));
            download(ctx, r);
            report("LeapfrogKDK::step x 50 == gvs_kdk_steps(50)", same(p.x, r.x) && same(p.vz, r.vz));
        }
        // 3. BarnesHut
        {
            Particles p = p0;
            p.clear_accelerations();
            BarnesHut bh(ctx, eps, 0.5);
            bh.compute_accelerations(p);
            Particles r = p0;
            upload(ctx, r, false);
            ctx.check(gvs_compute_forces(ctx.get(), GVS_ALGO_BH, GVS_PREC_FP64, eps, 0.5));
            download(ctx, r);
            report("BarnesHut::compute_accelerations == resident BH forces", same(p.ay, r.ay));
        }
        // 4. SPH drop-ins
        {
            EvrardCollapse ev;
            ev.n_particles = 1500;
            const Particles g0 = ev.generate();
            const double geps = ev.suggested_softening();
            Particles p = g0;
            BruteForce bf(ctx, geps);
            SphSolver sph(ctx);
            p.clear_accelerations();
            bf.compute_accelerations(p);
            sph.compute(p);
            double dtc = std::fmin(sph.compute_timestep(p), 1e-3);
            for (int s = 0; s < 3; ++s) dtc = std::fmin(step_with_sph(p, bf, sph, dtc), 1.5 * dtc);

            Particles r = g0;
            upload(ctx, r, false);
            ctx.check(gvs_compute_forces(ctx.get(), GVS_ALGO_DIRECT, GVS_PREC_FP64_EXACT, geps, 0.5));
            ctx.check(gvs_sph_compute(ctx.get(), &sph.params, nullptr, nullptr, nullptr, nullptr));
            double dtr = 0.0;
            ctx.check(gvs_sph_timestep(ctx.get(), &sph.params, &dtr));
            dtr = std::fmin(dtr, 1e-3);
            for (int s = 0; s < 3; ++s) {
                double nx = 0.0;
                ctx.check(gvs_sph_step(ctx.get(), &sph.params, GVS_ALGO_DIRECT, GVS_PREC_FP64_EXACT, geps, 0.5, dtr,
                                       &nx));
                dtr = std::fmin(nx, 1.5 * dtr);
            }
            download(ctx, r);
            report("SphSolver + step_with_sph x 3 == resident SPH steps",
                   dtc == dtr && same(p.x, r.x) && same(p.internal_energy, r.internal_energy) &&
                       same(p.density, r.density));
        }
    } catch (const Error &e) {
        std::printf("FAIL exception: %s\n", e.what());
        return 2;
    }
    return failures ? 1 : 0;
}
