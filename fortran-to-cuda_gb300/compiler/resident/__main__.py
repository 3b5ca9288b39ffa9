"""python -m compiler.resident APP.toml --output DIR [--variant V] [--fortran FC] [--prepare-only]

Prepares a resident build of a described application (entries spliced into its
selected procedures, directives expanded, CMake written) and builds it with its
native control when a Fortran compiler exists (the reference's CLI,
compiler/resident/__main__.py:18-65).
"""

from __future__ import annotations

import argparse
import json
import sys

from . import application, build


def main(argv=None) -> int:
    parser = argparse.ArgumentParser(prog="python -m compiler.resident", description=__doc__.splitlines()[0])
    parser.add_argument("description")
    parser.add_argument("--output", required=True)
    parser.add_argument("--variant")
    parser.add_argument("--fortran")
    parser.add_argument("--cmake", default="cmake")
    parser.add_argument("--jobs", type=int, default=8)
    parser.add_argument("--prepare-only", action="store_true")
    args = parser.parse_args(argv)
    try:
        app = application.load(args.description, args.variant)
        application.prepare(app, args.output)
    except application.DescriptionError as error:
        print(f"error: {error}", file=sys.stderr)
        return 2
    outcome = "prepared" if args.prepare_only else build.configure_and_build(args.output, args.fortran, args.cmake,
                                                                              args.jobs)
    print(json.dumps({"application": app.name, "entries": len(app.report["entries"]),
                      "nests": app.report["nests"], "directives": len(app.report["directives"]),
                      "outcome": outcome}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
