// Reference harness: drives the reference's own optimised solvers on given inputs.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled by oracle/Makefile (target `ref`)
// against the reference sources where they lie, into oracle/_ref/. It is never part
// of the shipped library; tests use it to pin the C restatement in
// oracle/swe_oracle.c and to generate the golden fixtures in tests/golden/.
//
// Reflecting walls run the reference's solver classes unmodified:
//   FastHLLMUSCLBathySolver         include/backend/serial/HPC/HPC_solver.hpp:88-482
//   FastHLLMUSCLBathyOpenMPSolver   include/backend/openmp/omp_solver.hpp
// Their private state (h_, hu_, hv_, B_, dt_) is reached with the usual
// `#define private public` test trick, so the inputs are injected bit-for-bit and
// the real rk3_step (HPC_solver.hpp:233-318) and apply_reflecting_bc (:320-371)
// run.  Adaptive dt calls the reference's compute_stable_dt (HPC_kernels.hpp:281-298)
// before every step.
//
// Transmissive (zero-gradient) walls do not exist in the reference. For them the
// harness calls the reference kernels (compute_x_fluxes, compute_y_fluxes,
// apply_divergence, enforce_positivity) in the order of HPC_solver.hpp:233-318,
// with the RK combines written as there, and a zero-gradient ghost copy in place
// of apply_reflecting_bc.
#include <bits/stdc++.h>

#define private public
#include "include/backend/serial/HPC/HPC_solver.hpp"
#include "include/backend/openmp/omp_solver.hpp"
#undef private

// ---- no-op I/O: the harness never writes NetCDF -------------------------------------
#include "netcdf_noop.cpp"

namespace {

SimulationConfig make_cfg(int Nx, int Ny, double Lx, double Ly, double cfl, int steps,
                          BackendType backend) {
    SimulationConfig cfg{};
    cfg.mesh.Lx = Lx;
    cfg.mesh.Ly = Ly;
    cfg.mesh.nG = 2;
    cfg.mesh.Nx = Nx;
    cfg.mesh.Ny = Ny;
    cfg.mesh.spatial_unit_x = cfg.mesh.spatial_unit_y = cfg.mesh.spatial_unit_h = "m";
    cfg.bathymetry.type = BathymetryType::Flat;
    cfg.bathymetry.b0 = 0.0;
    cfg.boundary.type = BoundaryType::ReflectingWalls;
    cfg.initial_condition.type = InitialConditionType::StillWater;
    cfg.initial_condition.h0 = 1.0;
    cfg.solver.reconstruction = ReconstructionType::MUSCL;
    cfg.solver.riemann = RiemannType::HLL;
    cfg.solver.time = TimeIntegratorType::SSPRK3;
    cfg.time.end_time = 1.0;
    cfg.time.time_steps = static_cast<std::size_t>(std::max(steps, 1));
    cfg.time.cfl = cfl;
    cfg.time.save_every = std::max(steps, 1);
    cfg.time.time_unit = "s";
    cfg.backend.type = backend;
    cfg.backend.threads = 1;
    cfg.output.path = "/dev/null";
    return cfg;
}

// Runs the reference solver class S on injected inputs (reflecting walls).
template <class S, class StableDt>
int run_class(S &s, int steps, double dt_fixed, double *h, double *hu, double *hv,
              const double *B, double *dt_log, double *t_out, StableDt stable_dt) {
    const std::size_t n = s.n_total_;
    std::copy(B, B + n, s.B_.begin());
    std::copy(h, h + n, s.h_.begin());
    std::copy(hu, hu + n, s.hu_.begin());
    std::copy(hv, hv + n, s.hv_.begin());
    s.apply_reflecting_bc(s.h_.data(), s.hu_.data(), s.hv_.data());
    double t = 0.0;
    for (int step = 0; step < steps; ++step) {
        if (dt_fixed > 0.0) {
            s.dt_ = dt_fixed;
        } else {
            s.dt_ = stable_dt(s.gv_, s.h_.data(), s.hu_.data(), s.hv_.data(), s.cfg_.time.cfl);
        }
        if (dt_log) dt_log[step] = s.dt_;
        s.rk3_step(static_cast<std::size_t>(step));
        t += s.dt_;
    }
    std::copy(s.h_.begin(), s.h_.end(), h);
    std::copy(s.hu_.begin(), s.hu_.end(), hu);
    std::copy(s.hv_.begin(), s.hv_.end(), hv);
    if (t_out) *t_out = t;
    return 0;
}

// Zero-gradient ghost fill: x-ghost rows for interior j, then y-ghost columns for
// all rows (the same sweep order as apply_reflecting_bc, HPC_solver.hpp:320-371).
void transmissive_bc(const fast_hll_muscl_bathy::GridView &gv, double *h, double *hu,
                     double *hv) {
    const int nG = gv.nG, Nx = gv.Nx, Ny = gv.Ny, s = gv.stride;
    for (int g = 0; g < nG; ++g) {
        const int iL = nG - 1 - g, iR = nG + Nx + g;
        for (int j = nG; j < nG + Ny; ++j) {
            const int kL = iL * s + j, kSL = nG * s + j;
            const int kR = iR * s + j, kSR = (nG + Nx - 1) * s + j;
            h[kL] = h[kSL];
            hu[kL] = hu[kSL];
            hv[kL] = hv[kSL];
            h[kR] = h[kSR];
            hu[kR] = hu[kSR];
            hv[kR] = hv[kSR];
        }
    }
    for (int g = 0; g < nG; ++g) {
        const int jB = nG - 1 - g, jT = nG + Ny + g;
        for (int i = 0; i < gv.Nx_total; ++i) {
            const int kB = i * s + jB, kSB = i * s + nG;
            const int kT = i * s + jT, kST = i * s + nG + Ny - 1;
            h[kB] = h[kSB];
            hu[kB] = hu[kSB];
            hv[kB] = hv[kSB];
            h[kT] = h[kST];
            hu[kT] = hu[kST];
            hv[kT] = hv[kST];
        }
    }
}

int run_transmissive(int Nx, int Ny, double Lx, double Ly, double cfl, int steps,
                     double dt_fixed, double *h, double *hu, double *hv, const double *B,
                     double *dt_log, double *t_out) {
    namespace fk = fast_hll_muscl_bathy;
    const Grid grid(Nx, Ny, Lx, Ly, 2);
    const fk::GridView gv{grid.Nx(),       grid.Ny(),       grid.nG(), grid.Nx_total(),
                          grid.Ny_total(), grid.Ny_total(), grid.dx(), grid.dy()};
    const std::size_t n = static_cast<std::size_t>(gv.Nx_total) * gv.Ny_total;
    std::vector<double> h1(n), hu1(n), hv1(n), h2(n), hu2(n), hv2(n), rh(n), rhu(n), rhv(n);
    std::vector<double> f[12];
    for (auto &a : f) a.assign(n, 0.0);
    auto rhs = [&](const double *a, const double *b, const double *c) {
        fk::compute_x_fluxes(gv, a, b, c, B, f[0].data(), f[1].data(), f[2].data(), f[3].data(),
                             f[4].data(), f[5].data());
        fk::compute_y_fluxes(gv, a, b, c, B, f[6].data(), f[7].data(), f[8].data(), f[9].data(),
                             f[10].data(), f[11].data());
        fk::apply_divergence(gv, f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data(),
                             f[5].data(), f[6].data(), f[7].data(), f[8].data(), f[9].data(),
                             f[10].data(), f[11].data(), rh.data(), rhu.data(), rhv.data());
    };
    transmissive_bc(gv, h, hu, hv);
    double t = 0.0;
    for (int step = 0; step < steps; ++step) {
        const double dt = dt_fixed > 0.0 ? dt_fixed : fk::compute_stable_dt(gv, h, hu, hv, cfl);
        if (dt_log) dt_log[step] = dt;
        transmissive_bc(gv, h, hu, hv);
        rhs(h, hu, hv);
        for (std::size_t k = 0; k < n; ++k) {
            h1[k] = h[k] + dt * rh[k];
            hu1[k] = hu[k] + dt * rhu[k];
            hv1[k] = hv[k] + dt * rhv[k];
        }
        fk::enforce_positivity(gv, h1.data(), hu1.data(), hv1.data());
        transmissive_bc(gv, h1.data(), hu1.data(), hv1.data());
        rhs(h1.data(), hu1.data(), hv1.data());
        for (std::size_t k = 0; k < n; ++k) {
            h2[k] = 0.75 * h[k] + 0.25 * (h1[k] + dt * rh[k]);
            hu2[k] = 0.75 * hu[k] + 0.25 * (hu1[k] + dt * rhu[k]);
            hv2[k] = 0.75 * hv[k] + 0.25 * (hv1[k] + dt * rhv[k]);
        }
        fk::enforce_positivity(gv, h2.data(), hu2.data(), hv2.data());
        transmissive_bc(gv, h2.data(), hu2.data(), hv2.data());
        rhs(h2.data(), hu2.data(), hv2.data());
        for (std::size_t k = 0; k < n; ++k) {
            h[k] = (1.0 / 3.0) * h[k] + (2.0 / 3.0) * (h2[k] + dt * rh[k]);
            hu[k] = (1.0 / 3.0) * hu[k] + (2.0 / 3.0) * (hu2[k] + dt * rhu[k]);
            hv[k] = (1.0 / 3.0) * hv[k] + (2.0 / 3.0) * (hv2[k] + dt * rhv[k]);
        }
        fk::enforce_positivity(gv, h, hu, hv);
        transmissive_bc(gv, h, hu, hv);
        t += dt;
    }
    if (t_out) *t_out = t;
    return 0;
}

} // namespace

extern "C" {

// Gravity this build of the harness was compiled with (reference constants::g).
double ref_gravity(void) { return constants::g; }

// Runs `steps` SSP-RK3 steps of the reference optimised path on full ghosted,
// row-major (k = i*(Ny+4) + j) arrays.  bc: 0 reflecting, 1 transmissive.
// solver: 0 HPC_solver (one thread), 1 omp_solver.  dt_fixed > 0 uses that dt for
// every step; otherwise dt = compute_stable_dt(U^n) before every step.
// Returns 0, 1 on a non-finite state (the reference's runtime_error), 2 otherwise.
int ref_run(int Nx, int Ny, double Lx, double Ly, double cfl, int bc, int solver, int steps,
            double dt_fixed, double *h, double *hu, double *hv, const double *B, double *dt_log,
            double *t_out) {
    try {
        if (bc == 1) {
            return run_transmissive(Nx, Ny, Lx, Ly, cfl, steps, dt_fixed, h, hu, hv, B, dt_log,
                                    t_out);
        }
        if (solver == 0) {
            FastHLLMUSCLBathySolver s(
                make_cfg(Nx, Ny, Lx, Ly, cfl, steps, BackendType::OptimizedSerial));
            return run_class(s, steps, dt_fixed, h, hu, hv, B, dt_log, t_out,
                             fast_hll_muscl_bathy::compute_stable_dt);
        }
        FastHLLMUSCLBathyOpenMPSolver s(make_cfg(Nx, Ny, Lx, Ly, cfl, steps, BackendType::OpenMP));
        return run_class(s, steps, dt_fixed, h, hu, hv, B, dt_log, t_out,
                         fast_hll_muscl_bathy_omp::compute_stable_dt);
    } catch (const std::runtime_error &e) {
        std::fprintf(stderr, "ref_run: %s\n", e.what());
        return std::strstr(e.what(), "non-finite") ? 1 : 2;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "ref_run: %s\n", e.what());
        return 2;
    }
}

// The reference's compute_stable_dt (HPC_kernels.hpp:281-298) on a ghosted state.
double ref_stable_dt(int Nx, int Ny, double Lx, double Ly, double cfl, const double *h,
                     const double *hu, const double *hv) {
    const Grid grid(Nx, Ny, Lx, Ly, 2);
    const fast_hll_muscl_bathy::GridView gv{grid.Nx(),       grid.Ny(),       grid.nG(),
                                            grid.Nx_total(), grid.Ny_total(), grid.Ny_total(),
                                            grid.dx(),       grid.dy()};
    return fast_hll_muscl_bathy::compute_stable_dt(gv, h, hu, hv, cfl);
}

} // extern "C"
