"""The CMake project of a prepared resident build (and its native control).

Two object libraries, as the reference's build (compiler/resident/build.py:53-112,
201-230): ``native`` from the unchanged sources and ``resident`` from the
prepared ones plus this library's Fortran modules (fort_scoped_memory,
fort_resident_domain, fort_resident_application and the entry interfaces),
linked against libf2c_gb300.so. Every language gets the strict numerical
options (-ffp-contract=off), except under --fast-fp, where, as in the
reference's build (compiler/resident/build.py:22,57-66), both builds drop them
and the resident objects are preprocessed with F2C_FAST_FP, so that the
residency domain opens its contexts under the fast-fp contract (the entries
then run the library's fast-fp kernels). One executable per [[executable]].
"""

from __future__ import annotations

import json
import shutil
import subprocess
from pathlib import Path

from .. import native

FORTRAN_MODULES = ("fort_scoped_memory.f90", "fort_resident_domain.f90", "fort_resident_application.f90",
                   "fort_shared_entries.f90")
STRICT = ("-ffp-contract=off",)


def _cmake_list(items) -> str:
    return " ".join(f'"{i}"' for i in items)


def write_cmake(app, output, fast_fp: bool = False) -> Path:
    output = Path(output)
    modules_dir = native.PACKAGE_ROOT / "fortran"
    options = list(app.build.get("fortran_options", [])) + ([] if fast_fp else list(STRICT)) + ["-cpp"]
    defines = [f"-D{d}" for d in app.defines]
    link = [x for x in app.build.get("link", []) if x != "OpenMP::OpenMP_Fortran"]
    libraries = list(app.build.get("libraries", []))
    program = app.program.name
    others = [s.name for s in app.sources if s.name != program]
    lines = [
        "cmake_minimum_required(VERSION 3.24)",
        f"project({app.name} LANGUAGES Fortran)",
        "find_package(OpenMP REQUIRED)",
        f'set(F2C_GB300_LIBRARY "{native.LIBRARY}")',
        f"set(F2C_FORTRAN_OPTIONS {_cmake_list(options + defines)})",
        "add_library(native_objects OBJECT " + _cmake_list(f"native/{s}" for s in others) + ")",
        "add_library(resident_objects OBJECT "
        + _cmake_list([*(str(modules_dir / m) for m in FORTRAN_MODULES), *(f"resident/{s}" for s in others)]) + ")",
        'set_target_properties(native_objects PROPERTIES Fortran_MODULE_DIRECTORY "${CMAKE_BINARY_DIR}/native-modules")',
        'set_target_properties(resident_objects PROPERTIES Fortran_MODULE_DIRECTORY '
        '"${CMAKE_BINARY_DIR}/resident-modules")',
        "target_compile_options(native_objects PRIVATE ${F2C_FORTRAN_OPTIONS})",
        "target_compile_options(resident_objects PRIVATE ${F2C_FORTRAN_OPTIONS})",
        *(["target_compile_definitions(resident_objects PRIVATE F2C_FAST_FP)"] if fast_fp else []),
        "target_link_libraries(native_objects PUBLIC OpenMP::OpenMP_Fortran " + " ".join(link) + ")",
        "target_link_libraries(resident_objects PUBLIC OpenMP::OpenMP_Fortran " + " ".join(link) + ")",
    ]
    for exe in app.executables:
        lib = "resident" if exe.library == "resident" else "native"
        lines += [f'add_executable({exe.name} "{lib}/{program}")',
                  f"target_compile_options({exe.name} PRIVATE ${{F2C_FORTRAN_OPTIONS}})",
                  f'target_include_directories({exe.name} PRIVATE "${{CMAKE_BINARY_DIR}}/{lib}-modules")',
                  f"target_link_libraries({exe.name} PRIVATE {lib}_objects {' '.join(libraries)}"
                  + (" ${F2C_GB300_LIBRARY}" if lib == "resident" else "") + ")"]
    (output / "CMakeLists.txt").write_text("\n".join(lines) + "\n")
    (output / "resident_build.json").write_text(json.dumps(app.report, indent=1, sort_keys=True) + "\n")
    return output / "CMakeLists.txt"


def configure_and_build(output, fortran: str | None, cmake: str = "cmake", jobs: int = 8) -> str:
    """Run CMake and the build when a Fortran compiler exists; otherwise say why not."""
    compiler = shutil.which(fortran) if fortran else None
    if compiler is None:
        for name in ("gfortran", "flang-new", "flang", "ifx"):
            compiler = shutil.which(name)
            if compiler:
                break
    if compiler is None:
        return "prepared; not built: no Fortran compiler on this machine"
    tool = shutil.which(cmake)
    if tool is None:
        return "prepared; not built: no cmake"
    output = Path(output)
    subprocess.run([tool, "-S", str(output), "-B", str(output / "build"), f"-DCMAKE_Fortran_COMPILER={compiler}"],
                   check=True)
    subprocess.run([tool, "--build", str(output / "build"), "-j", str(jobs)], check=True)
    return "built"
