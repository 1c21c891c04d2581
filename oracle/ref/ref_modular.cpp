// Reference harness for the modular solver: runs the reference's own
// SerialSolver<ReflectingWalls, Recon, Riemann, SSPRK3, Bathymetry>
// (include/backend/serial/serial_solver.hpp:105-524) on given inputs.
//
// TEST INFRASTRUCTURE ONLY. Compiled by oracle/Makefile (target `ref`) against the
// reference sources where they lie, into oracle/_ref/; tests use it to pin the C
// restatement in oracle/swe_modular.c.
//
// The solver class runs unmodified, run() included (its CFL guard, step loop,
// positivity checks and boundary refreshes).  Its private state (U_, B_, dt_, the
// integrator's dt_) is reached with the `#define private public` test trick, so that
// the inputs are injected bit-for-bit after construction.  NetCDF output goes to the
// no-op stub that ref_harness.cpp's translation unit defines.
#include <bits/stdc++.h>

#define private public
#include "include/backend/serial/serial_solver.hpp"
#undef private

namespace {

SimulationConfig modular_cfg(int Nx, int Ny, double Lx, double Ly, double cfl, int steps,
                             bool bathy) {
    SimulationConfig cfg{};
    cfg.mesh.Lx = Lx;
    cfg.mesh.Ly = Ly;
    cfg.mesh.nG = 2;
    cfg.mesh.Nx = Nx;
    cfg.mesh.Ny = Ny;
    cfg.mesh.spatial_unit_x = cfg.mesh.spatial_unit_y = cfg.mesh.spatial_unit_h = "m";
    cfg.bathymetry.type = bathy ? BathymetryType::Flat : BathymetryType::None;
    cfg.bathymetry.b0 = 0.0;
    cfg.boundary.type = BoundaryType::ReflectingWalls;
    cfg.initial_condition.type = InitialConditionType::StillWater;
    cfg.initial_condition.h0 = 1.0;
    cfg.solver.time = TimeIntegratorType::SSPRK3;
    cfg.time.end_time = 1.0;
    cfg.time.time_steps = static_cast<std::size_t>(std::max(steps, 1));
    cfg.time.cfl = cfl;
    cfg.time.save_every = std::max(steps, 1);
    cfg.time.time_unit = "s";
    cfg.backend.type = BackendType::Serial;
    cfg.backend.threads = 1;
    cfg.output.path = "/dev/null";
    return cfg;
}

int status_of(const std::runtime_error &e) {
    const std::string m = e.what();
    if (m.find("non-finite") != std::string::npos) return 1;
    if (m.find("HLL could not provide") != std::string::npos) return 2;
    if (m.find("Time step too large") != std::string::npos) return 3;
    return 4;
}

template <class R, class Rm, class Bt>
int run_one(int Nx, int Ny, double Lx, double Ly, double cfl, int steps, double dt, double *h,
            double *hu, double *hv, const double *B) {
    const SimulationConfig cfg = modular_cfg(Nx, Ny, Lx, Ly, cfl, steps, Bt::enabled);
    SerialSolver<ReflectingWalls, R, Rm, SSPRK3, Bt> s(cfg);
    const std::size_t n = static_cast<std::size_t>(Nx + 4) * static_cast<std::size_t>(Ny + 4);
    s.dt_ = dt;
    s.time_integrator_.dt_ = dt;
    s.steps_ = static_cast<std::size_t>(steps);
    s.save_every_ = static_cast<std::size_t>(std::max(steps, 1));
    if (Bt::enabled) {
        std::copy(B, B + n, s.B_.data());
        s.bc_.apply_BC(s.B_);  // as the constructor does after apply_bathymetry
    }
    std::copy(h, h + n, s.U_.h().data());
    std::copy(hu, hu + n, s.U_.hu().data());
    std::copy(hv, hv + n, s.U_.hv().data());
    int st = 0;
    try {
        s.run();
    } catch (const std::runtime_error &e) {
        st = status_of(e);
    }
    std::copy(s.U_.h().data(), s.U_.h().data() + n, h);
    std::copy(s.U_.hu().data(), s.U_.hu().data() + n, hu);
    std::copy(s.U_.hv().data(), s.U_.hv().data() + n, hv);
    return st;
}

template <class R, class Rm>
int run_bathy(int bathy, int Nx, int Ny, double Lx, double Ly, double cfl, int steps, double dt,
              double *h, double *hu, double *hv, const double *B) {
    return bathy ? run_one<R, Rm, Flat>(Nx, Ny, Lx, Ly, cfl, steps, dt, h, hu, hv, B)
                 : run_one<R, Rm, None>(Nx, Ny, Lx, Ly, cfl, steps, dt, h, hu, hv, B);
}

template <class R>
int run_riemann(int riemann, int bathy, int Nx, int Ny, double Lx, double Ly, double cfl,
                int steps, double dt, double *h, double *hu, double *hv, const double *B) {
    switch (riemann) {
        case 0: return run_bathy<R, HLL>(bathy, Nx, Ny, Lx, Ly, cfl, steps, dt, h, hu, hv, B);
        case 1: return run_bathy<R, Rusanov>(bathy, Nx, Ny, Lx, Ly, cfl, steps, dt, h, hu, hv, B);
        case 2: return run_bathy<R, ROE>(bathy, Nx, Ny, Lx, Ly, cfl, steps, dt, h, hu, hv, B);
        default: return -1;
    }
}

}  // namespace

extern "C" {

// recon 0: PiecewiseConst, 1: MUSCL; riemann 0: HLL, 1: Rusanov, 2: ROE; bathy 0: None,
// 1: Flat (enabled; B as given).  Returns 0, 1 non-finite, 2 HLL failure, 3 CFL guard,
// 4 other reference exception.
int ref_modular_run(int Nx, int Ny, double Lx, double Ly, double cfl, int recon, int riemann,
                    int bathy, int steps, double dt, double *h, double *hu, double *hv,
                    const double *B) {
    std::streambuf *old = std::cout.rdbuf(nullptr);  // run() prints its timing summary
    const int st = recon == 0
        ? run_riemann<PiecewiseConst>(riemann, bathy, Nx, Ny, Lx, Ly, cfl, steps, dt, h, hu, hv, B)
        : run_riemann<MUSCL>(riemann, bathy, Nx, Ny, Lx, Ly, cfl, steps, dt, h, hu, hv, B);
    std::fflush(stdout);  // its "INFO: Bathymetry enabled." line goes out with this call
    std::cout.rdbuf(old);
    return st;
}

// compute_stable_dt (include/solver_assembly/time_utils.hpp:14-38) on given arrays;
// returns 0, or 1 when it throws (h < 0).
int ref_modular_stable_dt(int Nx, int Ny, double Lx, double Ly, double cfl, const double *h,
                          const double *hu, const double *hv, double *out) {
    Grid grid(Nx, Ny, Lx, Ly, 2);
    State U(grid);
    const std::size_t n = static_cast<std::size_t>(Nx + 4) * static_cast<std::size_t>(Ny + 4);
    std::copy(h, h + n, U.h().data());
    std::copy(hu, hu + n, U.hu().data());
    std::copy(hv, hv + n, U.hv().data());
    try {
        *out = compute_stable_dt(U, grid, cfl);
    } catch (const std::runtime_error &) {
        return 1;
    }
    return 0;
}

}  // extern "C"
