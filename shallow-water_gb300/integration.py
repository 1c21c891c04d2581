"""Adds the GB300 backend to a copy of the reference's source tree.

The reference selects a backend at four sites (configs/config.hpp:7,
configs/simulation_config.cpp:11-18, configs/parse_config_helper.hpp:5-20,
include/solver_assembly/solver_assembly.hpp:17-120) plus a CMake option
(CMakeLists.txt:9-18).  :func:`patch_reference_tree` inserts a ``GB300`` value at each
site, in place, in a tree the caller owns (never the original checkout), so that
``[backend] type = "GB300"`` in simulation_config.toml constructs
``FastHLLMUSCLBathyGB300Solver`` (include/swe_gb300_solver.hpp) and calls ``run()``.
Each edit is anchored on a line of the reference and fails loudly if the anchor moved.
"""
from __future__ import annotations

import os

CASE_BLOCK = '''        case BackendType::GB300: {
#if USE_GB300
            // MUSCL + HLL over Flat / GaussHill bathymetry runs the fused scheme (as the
            // CUDA backend); every other [solver] / [bathymetry] choice runs the modular
            // scheme, as the Serial backend would (FastHLLMUSCLBathyGB300Solver decides).
            if (cfg_.boundary.type == BoundaryType::ReflectingWalls &&
                cfg_.solver.time == TimeIntegratorType::SSPRK3) {

                FastHLLMUSCLBathyGB300Solver solver(cfg_);
                solver.run();
                return;
            }

            throw std::runtime_error("Unsupported GB300 solver combination. "
                                     "The GB300 backend supports SSPRK3 + ReflectingWalls "
                                     "with any reconstruction, riemann and bathymetry.");
#else
            throw std::runtime_error(
                "GB300 backend was requested in simulation_config.toml, but this binary "
                "was built without GB300. Rebuild with ENABLE_GB300, or set "
                "[backend] type = \\"OptimizedSerial\\", \\"OpenMP\\", or \\"Serial\\".");
#endif
        }
'''

CMAKE_BLOCK = '''
# GB300 (sm_103a) backend: include/swe_gb300_solver.hpp over libswe_gb300.so
option(ENABLE_GB300 "Build the GB300 backend" OFF)
set(SWE_GB300_DIR "" CACHE PATH "Checkout of the GB300 backend (include/, shallow-water_gb300/)")
if(ENABLE_GB300)
    target_include_directories(swe_solver PRIVATE ${SWE_GB300_DIR}/include)
    target_link_libraries(swe_solver PRIVATE ${SWE_GB300_DIR}/shallow-water_gb300/libswe_gb300.so)
    target_compile_definitions(swe_solver PRIVATE USE_GB300=1)
else()
    target_compile_definitions(swe_solver PRIVATE USE_GB300=0)
endif()
'''

# (file, anchor, replacement) - the replacement keeps the anchor.
EDITS = [
    ("configs/config.hpp",
     "enum class BackendType { Serial, OptimizedSerial, OpenMP, CUDA, CUDA_4 };",
     "enum class BackendType { Serial, OptimizedSerial, OpenMP, CUDA, CUDA_4, GB300 };"),
    ("configs/simulation_config.cpp",
     '    if (s == "CUDA_4") return BackendType::CUDA_4;\n',
     '    if (s == "CUDA_4") return BackendType::CUDA_4;\n'
     '    if (s == "GB300") return BackendType::GB300;\n'),
    ("configs/parse_config_helper.hpp",
     '        return "CUDA_4";\n',
     '        return "CUDA_4";\n    case BackendType::GB300:\n        return "GB300";\n'),
    ("include/solver_assembly/solver_assembly.hpp",
     '#include "include/backend/cuda/four_gpu/cuda_solver_4gpu.hpp"\n#endif\n',
     '#include "include/backend/cuda/four_gpu/cuda_solver_4gpu.hpp"\n#endif\n\n'
     '#if USE_GB300\n#include "swe_gb300_solver.hpp"\n#endif\n'),
    ("include/solver_assembly/solver_assembly.hpp",
     "        case BackendType::CUDA_4: {\n",
     CASE_BLOCK + "        case BackendType::CUDA_4: {\n"),
]


def patch_reference_tree(root: str, cmake: bool = True) -> None:
    """Edits a writable copy of the reference tree at ``root`` in place."""
    for rel, anchor, repl in EDITS:
        path = os.path.join(root, rel)
        text = open(path).read()
        if text.count(anchor) != 1:
            raise RuntimeError(f"{rel}: anchor not found exactly once: {anchor!r}")
        os.chmod(path, 0o644)
        with open(path, "w") as f:
            f.write(text.replace(anchor, repl))
    if cmake:
        path = os.path.join(root, "CMakeLists.txt")
        os.chmod(path, 0o644)
        with open(path, "a") as f:
            f.write(CMAKE_BLOCK)
