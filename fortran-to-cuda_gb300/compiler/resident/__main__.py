"""python -m compiler.resident APP.toml --output DIR [--variant V] [--fortran FC] [--prepare-only | --build-prepared]

Prepares a resident build of a described application (entries spliced into its
selected procedures, directives expanded, CMake written) and builds it with its
native control when a Fortran compiler exists. The command line is the
reference's (compiler/resident/__main__.py:18-65): the same arguments are
accepted with the same meaning where they apply to this library. ``--cxx`` and
``--nvcc`` are not needed (the entries are prebuilt in libf2c_gb300.so) and are
only checked to exist when given; ``--architecture`` must name the one this
library is built for (103a); ``--fast-fp`` builds both trees without the strict
host option and opens the resident build's contexts under the fast-fp
numerical contract (the library's fast-fp kernels: FMA contraction and
regrouped sums, within 1e-12 of the strict result); ``--input`` trees belong to
applications outside the advection path and are refused. Errors print
``error: ...`` and exit with status 1.
"""

from __future__ import annotations

import argparse
import json
import shutil
import sys
from pathlib import Path

from . import application, build

ARCHITECTURES = {"103a", "103", "sm_103a", "sm_103", "compute_103a"}


def main(argv=None) -> int:
    parser = argparse.ArgumentParser(prog="python -m compiler.resident", description=__doc__.splitlines()[0])
    parser.add_argument("description", help="The application's TOML description")
    parser.add_argument("--input", action="append", default=[], metavar="NAME=PATH")
    parser.add_argument("--output", required=True, help="A new directory for the build")
    parser.add_argument("--variant", help="A variant of the description; its first by default")
    parser.add_argument("--fortran", help="A path, or a name to look up on PATH")
    parser.add_argument("--prepare-only", action="store_true", help="Write the resident sources, compile nothing")
    parser.add_argument("--build-prepared", action="store_true", help="Compile what an earlier run prepared")
    parser.add_argument("--cxx")
    parser.add_argument("--nvcc")
    parser.add_argument("--architecture")
    parser.add_argument("--cmake", default="cmake")
    parser.add_argument("--jobs", type=int, default=8)
    parser.add_argument("--fast-fp", action="store_true",
                        help="FMA contraction and regrouped sums instead of the strict numerical contract")
    args = parser.parse_args(argv)
    try:
        if args.jobs < 1:
            raise ValueError("jobs must be positive")
        if args.prepare_only and args.build_prepared:
            raise ValueError("choose preparation or building prepared sources")
        if args.input:
            raise ValueError("--input trees describe applications outside the advection path")
        if args.architecture and args.architecture.lower() not in ARCHITECTURES:
            raise ValueError(f"this library is built for sm_103a, not {args.architecture}")
        for tool in (args.cxx, args.nvcc):
            if tool and not shutil.which(tool):
                raise ValueError(f"{tool} not found")
        output = Path(args.output)
        if args.build_prepared:
            report = json.loads((output / "resident_build.json").read_text())
            name = report["application"]
        else:
            app = application.load(args.description, args.variant)
            application.prepare(app, output, fast_fp=args.fast_fp)
            report, name = app.report, app.name
        outcome = "prepared" if args.prepare_only else build.configure_and_build(output, args.fortran, args.cmake,
                                                                                  args.jobs)
    except (application.DescriptionError, ValueError, OSError, KeyError) as error:
        print(f"error: {error}", file=sys.stderr)
        return 1
    print(json.dumps({"application": name, "entries": len(report["entries"]), "nests": report["nests"],
                      "directives": len(report["directives"]), "outcome": outcome}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
