// FastHLLMUSCLBathyGB300Solver - the reference's backend-class contract over the C ABI.
//
// A drop-in beside FastHLLMUSCLBathySolver (include/backend/serial/HPC/HPC_solver.hpp:88)
// and FastHLLMUSCLBathyOpenMPSolver (include/backend/openmp/omp_solver.hpp) for the
// reference's SolverAssembly switch (include/solver_assembly/solver_assembly.hpp:36-120).
// It is compiled inside the reference's source tree (its include root on the path),
// because the host-side set-up is the reference's own: SimulationConfig, Grid, State,
// Array2D, apply_bathymetry, apply_initial_condition, NetCDFWriter and the sanity
// checks.  The hot path (MUSCL + hydrostatic reconstruction + HLL + SSP-RK3 + walls +
// CFL reduction) runs on the GPU through include/swe_gb300.h.
//
// Contract kept from the reference classes (cuda_solver.hpp:109-230):
//   * explicit ctor(const SimulationConfig&): bathymetry -> scalar wall ghosts -> initial
//     condition -> sanity-check initialisation; the device state is allocated and uploaded.
//   * run(): the CFL guard once (throws "Time step too large: ..."), a snapshot at t = 0,
//     fixed dt = end_time / time_steps, a snapshot and the sanity checks every save_every
//     steps and at the end, the ETA line, a timing summary.
//   * non-copyable, RAII device memory, errors as std::runtime_error.
//
// Scheme: with [solver] MUSCL + HLL and Flat or GaussHill bathymetry - the combination
// the reference's optimised backends run - the class uses the fused scheme, bitwise
// FastHLLMUSCLBathySolver (HPC_solver.hpp).  Every other [solver] reconstruction /
// riemann and [bathymetry] choice runs the modular scheme, bitwise the reference's
// SerialSolver for that combination (serial_solver.hpp; the Serial backend's dispatch,
// solver_assembly.hpp:330-490), where the optimised backends would ignore the setting.
//
// With SWE_GB300_NATIVE_OUTPUT=1 the snapshots go through the library's own NetCDF
// writer (swe_snapshot_*) instead of the reference's NetCDFWriter: each record is packed
// on the GPU and written by a background thread while the run continues, so an output
// step no longer stops the solver for a download.  The file holds the same dimensions,
// variables, attributes and values (classic encoding instead of netCDF-4).  The state
// is then downloaded only for the sanity checks, when any are configured.
#pragma once

#ifndef SWE_GB300_NATIVE_OUTPUT
#define SWE_GB300_NATIVE_OUTPUT 0
#endif

#include "configs/config.hpp"
#include "configs/parse_config_helper.hpp"
#include "include/bathymetry/apply_bathymetry.hpp"
#include "include/core/array2D.hpp"
#include "include/core/grid.hpp"
#include "include/core/state.hpp"
#include "include/initial_condition/apply_initial_condition.hpp"
#include "include/io/netCDF_writer.hpp"
#include "include/io/sanity_checks_netdcdf_writer.hpp"
#include "include/solver_assembly/time_utils.hpp"
#include "tests/sanity_checks/sanity_checks.hpp"

#include "swe_gb300.h"

#include <algorithm>
#include <chrono>
#include <cstddef>
#include <iomanip>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

class FastHLLMUSCLBathyGB300Solver {
  public:
    explicit FastHLLMUSCLBathyGB300Solver(const SimulationConfig &cfg)
        : cfg_(cfg), grid_(cfg.mesh.Nx, cfg.mesh.Ny, cfg.mesh.Lx, cfg.mesh.Ly, cfg.mesh.nG),
          dt_(cfg.time.end_time / static_cast<double>(cfg.time.time_steps)),
          steps_(cfg.time.time_steps), save_every_(static_cast<std::size_t>(cfg.time.save_every)),
          n_total_(static_cast<std::size_t>(grid_.Nx_total()) *
                   static_cast<std::size_t>(grid_.Ny_total())),
          h_(n_total_), hu_(n_total_), hv_(n_total_), B_(n_total_), io_state_(grid_),
          io_bathy_(grid_.Nx_total(), grid_.Ny_total()),
#if !SWE_GB300_NATIVE_OUTPUT
          writer_(cfg.output.path.string(), grid_, cfg.mesh.spatial_unit_x, cfg.mesh.spatial_unit_y,
                  cfg.mesh.spatial_unit_h, cfg.time.time_unit, cfg.time.save_every),
#endif
          sanity_checks_(make_sanity_checks(cfg)), sanity_writer_(make_sanity_writer(cfg, dt_)) {
        if (grid_.nG() != 2) {
            throw std::runtime_error("FastHLLMUSCLBathyGB300Solver requires nG == 2 for MUSCL.");
        }

        swe_params p;
        swe_params_default(&p);
        if (!fused(cfg_)) {
            p.scheme = SWE_SCHEME_MODULAR;
            p.reconstruction = cfg_.solver.reconstruction == ReconstructionType::MUSCL
                                   ? SWE_RECON_MUSCL : SWE_RECON_PIECEWISE_CONST;
            p.riemann = cfg_.solver.riemann == RiemannType::HLL       ? SWE_RIEMANN_HLL
                        : cfg_.solver.riemann == RiemannType::Rusanov ? SWE_RIEMANN_RUSANOV
                                                                      : SWE_RIEMANN_ROE;
            p.bathymetry = cfg_.bathymetry.type != BathymetryType::None;
        }
        p.Nx = grid_.Nx();
        p.Ny = grid_.Ny();
        p.nG = grid_.nG();
        p.Lx = grid_.Lx();
        p.Ly = grid_.Ly();
        p.g = constants::g;
        p.cfl = cfg.time.cfl;
        p.bc = SWE_BC_REFLECTING;  // BoundaryType has ReflectingWalls only (configs/config.hpp:9)
        p.precision = SWE_PRECISION_FP64;
        check(swe_create(&p, &ctx_), "swe_create");

        Array2D B_tmp(grid_.Nx_total(), grid_.Ny_total());
        apply_bathymetry(cfg_, grid_, B_tmp);
        scalar_wall_ghosts(B_tmp.data());
        std::copy(B_tmp.data(), B_tmp.data() + B_tmp.size(), B_.begin());
        std::copy(B_.begin(), B_.end(), io_bathy_.data());
#if SWE_GB300_NATIVE_OUTPUT
        open_native_output();
#else
        writer_.write_bathymetry(io_bathy_);
#endif

        State U_tmp(grid_);
        apply_initial_condition(cfg_, grid_, U_tmp);
        std::copy(U_tmp.h().data(), U_tmp.h().data() + n_total_, h_.begin());
        std::copy(U_tmp.hu().data(), U_tmp.hu().data() + n_total_, hu_.begin());
        std::copy(U_tmp.hv().data(), U_tmp.hv().data() + n_total_, hv_.begin());

        // Upload, then download once: the library fills the wall ghosts exactly as
        // apply_reflecting_bc does, so the host copy matches the reference's after its ctor.
        check(swe_upload(ctx_, h_.data(), hu_.data(), hv_.data(), B_.data()), "swe_upload");
        check(swe_download(ctx_, h_.data(), hu_.data(), hv_.data()), "swe_download");

        for (auto &c : sanity_checks_) {
            fill_io_state();
            c->initialize(io_state_, grid_);
        }
    }

    ~FastHLLMUSCLBathyGB300Solver() {
#if SWE_GB300_NATIVE_OUTPUT
        swe_snapshot_destroy(snap_);
#endif
        swe_destroy(ctx_);
    }

    FastHLLMUSCLBathyGB300Solver(const FastHLLMUSCLBathyGB300Solver &) = delete;
    FastHLLMUSCLBathyGB300Solver &operator=(const FastHLLMUSCLBathyGB300Solver &) = delete;

    void run() {
        std::cout << std::unitbuf;
        std::cerr << std::unitbuf;
        if (fused(cfg_))
            std::cout << "INFO: GB300 fused-stage solver active\n";
        else
            std::cout << "INFO: GB300 modular solver active (" << reconstruction_name(cfg_)
                      << " + " << riemann_name(cfg_) << ")\n";

        double dt_stable = 0.0;
        {
            const auto start = Clock::now();
            check(swe_stable_dt(ctx_, &dt_stable), "swe_stable_dt");
            cfl_check_s_ += seconds_since(start);
        }
        if (dt_ > dt_stable) {
            throw std::runtime_error("Time step too large: dt = " + std::to_string(dt_) +
                                     ", but CFL requires dt <= " + std::to_string(dt_stable));
        }

        double time = 0.0;
        const std::size_t eta_probe = std::min<std::size_t>(100, steps_);
        bool eta_printed = !cfg_.output.compute_eta;
        const auto start_wall = Clock::now();

        snapshot(time, true);
        sanity(time, 0);

        std::size_t done = 0;
        while (done < steps_) {
            // Advance to the next output step or ETA probe in one call (device-resident).
            std::size_t next = std::min(steps_, (done / save_every_ + 1) * save_every_);
            if (!eta_printed && eta_probe > done) next = std::min(next, eta_probe);
            const int n = static_cast<int>(next - done);
            {
                const auto start = Clock::now();
                check(swe_step(ctx_, n, dt_, &time), "swe_step");
                step_s_ += seconds_since(start);
            }
            done = next;
            if (!eta_printed && done == eta_probe) {
                const double elapsed = seconds_since(start_wall);
                std::cout << "ETA = " << format_duration(estimate_eta_seconds(done, steps_, elapsed))
                          << '\n';
                eta_printed = true;
            }
            if (done % save_every_ == 0 || done == steps_) {
                snapshot(time, false);
                sanity(time, done);
            }
        }
#if SWE_GB300_NATIVE_OUTPUT
        {
            const auto start = Clock::now();
            check_snap(swe_snapshot_close(snap_), "swe_snapshot_close");
            output_s_ += seconds_since(start);
        }
#endif
        print_summary(done);
    }

  private:
    using Clock = std::chrono::steady_clock;
    static double seconds_since(Clock::time_point t) {
        return std::chrono::duration<double>(Clock::now() - t).count();
    }

    void check(int status, const char *what) const {
        if (status == SWE_OK) return;
        std::string msg = std::string("GB300 backend: ") + what + ": " + swe_status_string(status);
        if (ctx_ && swe_last_error(ctx_)[0]) msg += std::string(" (") + swe_last_error(ctx_) + ")";
        // the modular scheme reports the Serial backend's own messages ("non-finite state
        // detected in positivity correction", "HLL could not provide dissipation speed.")
        if (status == SWE_ERR_NONFINITE)
            msg = fused(cfg_) ? std::string("non-finite state detected in GB300 solver")
                              : std::string(swe_last_error(ctx_));
        throw std::runtime_error(msg);
    }

    // apply_scalar_reflecting_bc (HPC_solver.hpp:373-404): mirror copies of B into ghosts.
    void scalar_wall_ghosts(double *a) const {
        const int nG = grid_.nG(), Nx = grid_.Nx(), Ny = grid_.Ny(), s = grid_.Ny_total();
        for (int g = 0; g < nG; ++g) {
            for (int j = nG; j < nG + Ny; ++j) {
                a[(nG - 1 - g) * s + j] = a[(nG + g) * s + j];
                a[(nG + Nx + g) * s + j] = a[(nG + Nx - 1 - g) * s + j];
            }
        }
        for (int g = 0; g < nG; ++g) {
            for (int i = 0; i < grid_.Nx_total(); ++i) {
                a[i * s + (nG - 1 - g)] = a[i * s + (nG + g)];
                a[i * s + (nG + Ny + g)] = a[i * s + (nG + Ny - 1 - g)];
            }
        }
    }

    void fill_io_state() {
        std::copy(h_.begin(), h_.end(), io_state_.h().data());
        std::copy(hu_.begin(), hu_.end(), io_state_.hu().data());
        std::copy(hv_.begin(), hv_.end(), io_state_.hv().data());
    }

#if SWE_GB300_NATIVE_OUTPUT
    void check_snap(int status, const char *what) const {
        if (status == SWE_OK) return;
        throw std::runtime_error(std::string("GB300 backend: ") + what + ": " +
                                 swe_status_string(status) + " (" +
                                 swe_snapshot_last_error(snap_) + ")");
    }

    // The NetCDFWriter constructor and write_bathymetry (netCDF_writer.cpp:10-27,85-98).
    void open_native_output() {
        swe_snapshot_params sp{};
        sp.Nx = grid_.Nx();
        sp.Ny = grid_.Ny();
        sp.dx = grid_.dx();
        sp.dy = grid_.dy();
        sp.unit_x = cfg_.mesh.spatial_unit_x.c_str();
        sp.unit_y = cfg_.mesh.spatial_unit_y.c_str();
        sp.unit_h = cfg_.mesh.spatial_unit_h.c_str();
        sp.unit_time = cfg_.time.time_unit.c_str();
        sp.save_every = cfg_.time.save_every;
        const std::string path = cfg_.output.path.string();
        const int st = swe_snapshot_open(path.c_str(), &sp, &snap_);
        if (st != SWE_OK)
            throw std::runtime_error("GB300 backend: cannot create " + path + ": " +
                                     swe_status_string(st));
        check_snap(swe_snapshot_bathymetry(snap_, B_.data()), "swe_snapshot_bathymetry");
    }

    // The device state goes to the file from the GPU; the host copy is refreshed only when
    // a sanity check needs it.
    void snapshot(double time, bool first) {
        const auto start = Clock::now();
        if (first) {
            const std::string backend = backend_name_from_cfg(cfg_);
            const std::string bathy = bathymetry_name_from_cfg(cfg_);
            check_snap(swe_snapshot_metadata(snap_, dt_, backend.c_str(),
                                             riemann_name(cfg_).c_str(),
                                             reconstruction_name(cfg_).c_str(), "SSPRK3",
                                             "Reflecting Walls", bathy.c_str()),
                       "swe_snapshot_metadata");
        }
        check_snap(swe_snapshot_write(snap_, ctx_, time), "swe_snapshot_write");
        host_stale_ = !first;
        output_s_ += seconds_since(start);
    }
#else
    void snapshot(double time, bool first) {
        const auto start = Clock::now();
        if (!first) check(swe_download(ctx_, h_.data(), hu_.data(), hv_.data()), "swe_download");
        fill_io_state();
        if (first) {
            writer_.write_snapshot(io_state_, time, dt_, backend_name_from_cfg(cfg_),
                                   riemann_name(cfg_), reconstruction_name(cfg_), "SSPRK3",
                                   "Reflecting Walls", bathymetry_name_from_cfg(cfg_));
        } else {
            writer_.write_snapshot(io_state_, time);
        }
        output_s_ += seconds_since(start);
    }
#endif

    void sanity(double time, std::size_t step) {
        if (sanity_checks_.empty()) return;
        const auto start = Clock::now();
        if (host_stale_) {
            check(swe_download(ctx_, h_.data(), hu_.data(), hv_.data()), "swe_download");
            host_stale_ = false;
        }
        fill_io_state();
        for (auto &c : sanity_checks_) c->evaluate(io_state_, grid_, time, step, sanity_writer_.get());
        sanity_s_ += seconds_since(start);
    }

    static std::unique_ptr<SanityCheckNetCDFWriter> make_sanity_writer(const SimulationConfig &cfg,
                                                                       double dt) {
        if (!cfg.sanity_checks.debug) return nullptr;
        if (cfg.sanity_checks.output_path.empty()) {
            throw std::runtime_error(
                "sanity_checks.output_path must be set if debug mode is enabled");
        }
        return std::make_unique<SanityCheckNetCDFWriter>(
            cfg.sanity_checks.output_path.string(), cfg.time.time_unit, cfg.mesh.spatial_unit_h,
            cfg.time.save_every, dt, backend_name_from_cfg(cfg), riemann_name(cfg),
            reconstruction_name(cfg), "SSPRK3", "Reflecting Walls", bathymetry_name_from_cfg(cfg));
    }

    // The combination the optimised backends run (solver_assembly.hpp:50-117).
    static bool fused(const SimulationConfig &cfg) {
        return cfg.solver.reconstruction == ReconstructionType::MUSCL &&
               cfg.solver.riemann == RiemannType::HLL &&
               (cfg.bathymetry.type == BathymetryType::Flat ||
                cfg.bathymetry.type == BathymetryType::GaussHill);
    }
    // SerialSolver's riemann_name_static / reconstruction_name_static (serial_solver.hpp:
    // 397-418).
    static std::string riemann_name(const SimulationConfig &cfg) {
        switch (cfg.solver.riemann) {
            case RiemannType::Rusanov: return "Rusanov";
            case RiemannType::HLL: return "HLL";
            case RiemannType::ROE: return "ROE";
        }
        return "UnknownRiemann";
    }
    static std::string reconstruction_name(const SimulationConfig &cfg) {
        return cfg.solver.reconstruction == ReconstructionType::MUSCL ? "MUSCL" : "PiecewiseConst";
    }

    void print_summary(std::size_t steps) const {
        double dev_ms = 0.0;
        swe_last_step_ms(ctx_, &dev_ms);
        const double total = step_s_ + output_s_ + sanity_s_;
        std::cout << "\n========== GB300 solver timing summary ==========" << '\n';
        std::cout << "time steps           : " << steps << '\n';
        std::cout << "CFL check            : " << cfl_check_s_ << " s" << '\n';
        std::cout << "measured solver time : " << total << " s" << '\n';
        std::cout << std::fixed << std::setprecision(6);
        std::cout << std::left << std::setw(24) << "gpu rk3 steps" << std::right << std::setw(12)
                  << step_s_ << " s\n";
        std::cout << std::left << std::setw(24) << "output" << std::right << std::setw(12)
                  << output_s_ << " s\n";
        std::cout << std::left << std::setw(24) << "sanity checks" << std::right << std::setw(12)
                  << sanity_s_ << " s\n";
        std::cout << "=================================================\n";
    }

    const SimulationConfig cfg_;
    Grid grid_;
    double dt_{};
    std::size_t steps_{};
    std::size_t save_every_{};
    std::size_t n_total_{};
    std::vector<double> h_, hu_, hv_, B_;
    State io_state_;
    Array2D io_bathy_;
#if SWE_GB300_NATIVE_OUTPUT
    swe_snapshot *snap_ = nullptr;
#else
    NetCDFWriter writer_;
#endif
    bool host_stale_ = false;  // h_, hu_, hv_ behind the device state
    std::vector<std::unique_ptr<SanityCheck>> sanity_checks_;
    std::unique_ptr<SanityCheckNetCDFWriter> sanity_writer_;
    swe_ctx *ctx_ = nullptr;
    double cfl_check_s_ = 0.0, step_s_ = 0.0, output_s_ = 0.0, sanity_s_ = 0.0;
};
