"""The resident build surface: TOML description, procedure splice, !$fort directives, CMake (CPU only).

Follows the reference's own surface tests (tests/test_resident_directives.py,
tests/test_resident_application.py): directives expand to calls on the
application's residency object, malformed ones are refused with the line,
selected procedures get a call block that falls back to the original
statements, and a described application prepares into resident and native
source trees with one build. The Fortran produced is checked structurally
here; no Fortran compiler exists on these machines to compile it.
"""

import json
import re
from pathlib import Path

import pytest

from compiler import emission
from compiler.resident import __main__ as cli
from compiler.resident import application, directives, fortran, splice

from oracle.build_ref import REFERENCE  # noqa: E402  (the reference checkout, when this machine has one)

CDU_TOML = REFERENCE / "benchmarks" / "cdu" / "cdu.toml"

SYNTHETIC = """\
! kernels
module MomentumAdvection
  implicit none
  private
  integer, parameter :: knd = kind(1.0d0)
contains

  ! kernel
  subroutine set(arr, val, Unx, Uny, &
                 Unz)
    real(knd), contiguous, intent(out) :: arr(:,:,:)
    real(knd), intent(in) :: val
    integer, intent(in) :: Unx, Uny, Unz
    integer :: i, j, k

    !$OMP PARALLEL DO PRIVATE(i, j)
    do k = 2, Unz + 1
      do j = 2, Uny + 1
        do i = 2, Unx + 1
          arr(i,j,k) = val
        end do
      end do
    end do
    !$OMP END PARALLEL DO
  end subroutine set

  pure recursive function helper(n) result(r)
    integer, intent(in) :: n
    integer :: r
    r = n + 1
  contains
    pure function inner(x) result(y)
      integer, intent(in) :: x
      integer :: y
      y = x
    end function inner
  end function helper
end module MomentumAdvection
"""


def _balanced(text: str):
    blocks = ends = ifs = endifs = 0
    for line in text.splitlines():
        code = line.split("!", 1)[0].strip().lower()
        blocks += code == "block"
        ends += code == "end block"
        ifs += bool(re.match(r"if\s*\(.*\)\s*then$", code))
        endifs += code in ("endif", "end if")
    assert blocks == ends and ifs == endifs, (blocks, ends, ifs, endifs)


def test_procedure_finder_locates_executable_parts():
    found = {p.qualified: p for p in fortran.procedures(SYNTHETIC)}
    assert set(found) == {"momentumadvection::set", "momentumadvection::helper", "momentumadvection::inner"}
    lines = SYNTHETIC.splitlines()
    s = found["momentumadvection::set"]
    assert lines[s.header].strip().startswith("subroutine set(")
    assert lines[s.body].strip() == "!$OMP PARALLEL DO PRIVATE(i, j)"
    assert lines[s.end].strip() == "end subroutine set"
    h = found["momentumadvection::helper"]
    assert lines[h.body].strip() == "r = n + 1"
    assert lines[h.end].strip() == "contains"
    inner = found["momentumadvection::inner"]                # an internal procedure is a unit of its own
    assert (lines[inner.body].strip(), lines[inner.end].strip()) == ("y = x", "end function inner")


@pytest.mark.parametrize("line, call", [
    ("!$fort enter", "call resident%begin_epoch(int(0, c_int))"),
    ("!$fort enter budget(2_8**30) device(1)", "call resident%begin_epoch(int(1, c_int), int(2_8**30, c_size_t))"),
    ("!$fort leave", "if (resident%active) call resident%end_epoch()"),
    ("!$fort close", "call resident%close()"),
    ("!$fort publish if(step == n)", "if (resident%active .and. (step == n)) call resident%publish()"),
    ("!$fort active(on_device)", "on_device = resident%active"),
    ("!$fort release(tmp, work%buf)", "call resident%release_real(work%buf)"),
])
def test_directives_expand_to_residency_calls(line, call):
    text, records = directives.expand("program p\n    " + line + "\nend program p\n", origin="p")
    assert call in text
    assert "!$fort" not in text
    assert records[0]["line"] == 2
    _balanced(text)


def test_observe_binds_and_observes_named_arrays():
    text, _ = directives.expand("  !$fort observe(U, V) if(mod(step, 10) == 0)\n", origin="main")
    assert "integer(c_int64_t) :: fort_observed(2)" in text
    assert "fort_observed(2) = resident%bind(V, lbound(V), .true., origin='main::v')" in text
    assert "if (resident%active .and. (mod(step, 10) == 0)) then" in text
    assert "call resident%observe(fort_observed)" in text


DOMAIN = directives.Domain("my_state", "flow", "require", prefix="app")


def _expand(line):
    """One directive between two statements, expanded on the domain ``flow`` of module ``my_state``."""
    text, records = directives.expand("  x = 1\n" + line + "\n  y = 2\n", DOMAIN, origin="unit")
    assert text.startswith("  x = 1\n") and text.endswith("  y = 2\n")
    return text[len("  x = 1\n"):-len("  y = 2\n")], records


def test_text_without_directives_is_unchanged():
    source = "  !$omp parallel do\n  ! $fort is not a directive\n  a = '!$fort publish'\n  !$fortran x\n"
    assert directives.expand(source, DOMAIN) == (source, [])


def test_enter_starts_an_epoch_once_under_its_condition():
    block, records = _expand("    !$FORT enter budget(2*1024**3) if(supported() .and. (n > 1)) device(gpu)")
    assert block == ("    block\n"
                     "      use, intrinsic :: iso_c_binding\n"
                     "      use my_state, only: flow\n"
                     "      if (.not. flow%active) then\n"
                     "        if (supported() .and. (n > 1)) call flow%begin_epoch(int(gpu, c_int), "
                     "int(2*1024**3, c_size_t))\n"
                     "      endif\n"
                     "    end block\n")
    assert records == [{"line": 2, "directive": "enter", "arrays": [],
                        "clauses": {"budget": "2*1024**3", "if": "supported() .and. (n > 1)", "device": "gpu"}}]
    unconditional, _ = _expand("!$fort enter budget(1024)")
    assert "  if (.not. flow%active) then\n    call flow%begin_epoch(int(0, c_int), int(1024, c_size_t))\n" \
        in unconditional
    assert "    call flow%begin_epoch(int(0, c_int))\n" in _expand("!$fort enter")[0]  # the free device memory


def test_active_tells_the_source_and_annotations_generate_nothing():
    block, records = _expand("    !$fort active(on_device)")
    assert "      on_device = flow%active\n" in block
    assert records[0]["directive"] == "active"
    text, records = directives.expand("  do i = 1, n\n    !$fort host\n    s = s + a(i)\n  end do\n"
                                      "  !$fort reduction(+: s) private(i)\n", DOMAIN)
    assert text == "  do i = 1, n\n    s = s + a(i)\n  end do\n"
    assert [r["directive"] for r in records] == ["host", "reduction"]


def test_leave_close_and_publish_act_on_the_whole_domain():
    assert "if (flow%active) call flow%end_epoch()" in _expand("!$fort leave")[0]
    assert "  call flow%close()\n" in _expand("!$fort close")[0]  # also valid when no epoch ever began
    assert "if (flow%active) call flow%publish()" in _expand("!$fort publish")[0]
    assert "if (flow%active .and. (count > 0)) call flow%publish()" in _expand("!$fort publish if(count > 0)")[0]


def test_observe_binds_the_named_arrays_and_keeps_their_device_copies():
    block, records = _expand("  !$fort observe(U, state%pressure) if(mode == 2)")
    assert block == ("  block\n"
                     "    use, intrinsic :: iso_c_binding\n"
                     "    use my_state, only: flow\n"
                     "    integer(c_int64_t) :: app_observed(2)\n"
                     "    if (flow%active .and. (mode == 2)) then\n"
                     "      app_observed(1) = flow%bind(U, lbound(U), .true., origin='unit::u')\n"
                     "      app_observed(2) = flow%bind(state%pressure, lbound(state%pressure), .true., "
                     "origin='unit::state%pressure')\n"
                     "      call flow%observe(app_observed)\n"
                     "    endif\n"
                     "  end block\n")
    assert records[0]["arrays"] == ["U", "state%pressure"]


def test_observe_brings_one_field_of_an_array_of_derived_type_back():
    block, records = _expand("!$fort observe(points(:)%seen, u) if(ready)")
    assert block == ("block\n"
                     "  use, intrinsic :: iso_c_binding\n"
                     "  use my_state, only: flow\n"
                     "  integer(c_int64_t) :: app_observed(1)\n"
                     "  if (flow%active .and. (ready)) then\n"
                     "    app_observed(1) = flow%bind(u, lbound(u), .true., origin='unit::u')\n"
                     "    call flow%observe(app_observed)\n"
                     "    if (size(points) > 0) call flow%observe_field(c_loc(points(lbound(points,1))%seen))\n"
                     "  endif\n"
                     "end block\n")
    assert records[0]["arrays"] == ["points(:)%seen", "u"]
    assert "app_observed" not in _expand("!$fort observe(points(:)%seen)")[0]
    with pytest.raises(ValueError, match="takes array names, not expressions"):
        directives.expand("!$fort release(points(:)%seen)\n", DOMAIN)


def test_release_retires_temporaries_without_bringing_them_back():
    block, _ = _expand("!$fort release(tmp, work)")
    assert "if (flow%active) then\n    call flow%release_real(tmp)\n    call flow%release_real(work)\n  endif" in block


@pytest.mark.parametrize("line, message", [
    ("!$fort", "Empty residency directive on line 2"),
    ("!$fort sync", "Unknown residency directive on line 2: sync"),
    ("!$fort enter budget(1) when(x)", "Unsupported clause"),
    ("!$fort enter budget(1) if(a", "Unbalanced parentheses"),
    ("!$fort publish if", "Unsupported clause"),
    ("!$fort leave(a)", "takes no arguments"),
    ("!$fort leave if(x)", "Unsupported clause"),
    ("!$fort close(U)", "takes no arguments"),
    ("!$fort observe", "needs a list of arrays"),
    ("!$fort observe(a(1:n))", "takes array names, not expressions"),
    ("!$fort release(a+b)", "takes array names, not expressions"),
    ("!$fort publish, if(x)", "Malformed residency directive"),
    ("!$fort host(a)", "Malformed"),
    ("!$fort reduction", "Malformed"),
    ("!$fort reduction(s)", "Malformed"),
    ("!$fort active", "needs a list"),
    ("!$fort active(a, b)", "takes one logical variable"),
])
def test_malformed_directives_are_refused_with_their_line(line, message):
    with pytest.raises(directives.DirectiveError, match=message) as info:
        directives.expand("  x = 1\n" + line + "\n", DOMAIN)
    assert "line 2" in str(info.value)


def test_splice_calls_the_entry_and_keeps_the_original_statements():
    text, done = splice.splice(SYNTHETIC, ["momentumadvection::*"])
    entry = emission.entry_for("MomentumAdvection::set")
    assert [(d.procedure, d.entry, d.nests) for d in done] == [("momentumadvection::set", entry.symbol, 1)]
    assert f"use {entry.fortran_module}, only: fort_device_run => run" in text
    call = re.search(r"fort_status = fort_device_run\((.*?)\)\n", text, re.S).group(1)
    args = [a.strip(" &\n") for a in call.split(",")]
    assert args == ["resident%context", "FORT_SCOPE_GPU", "fort_handle_arr", "val", "Unx", "Uny", "Unz"]
    # the fallback holds the original loop nest, unchanged
    fallback = text[text.index("if (.not. fort_resident) then"):]
    assert "          arr(i,j,k) = val" in fallback
    assert fallback.index("call resident%publish()") < fallback.index("arr(i,j,k) = val")
    # the helper has no template and is left alone
    assert "r = n + 1\n  contains" in text
    _balanced(text)


def test_call_block_arguments_follow_the_generated_interfaces():
    """Every spliceable entry's call passes what its Fortran interface declares, in that order."""
    interfaces = (Path(emission.__file__).parents[2] / "fortran" / "fort_shared_entries.f90").read_text()
    for entry in emission.registry():
        block = splice.call_block(entry, "")
        call = re.search(r"fort_status = fort_device_run\((.*?)\)\n", block, re.S).group(1)
        args = [a.strip(" &\n").lower() for a in call.split(",")]
        module = interfaces[interfaces.index(f"module {entry.fortran_module}\n"):]
        header = re.search(r"function run\((.*?)\) bind", module, re.S).group(1)
        declared = [a.strip(" &\n") for a in header.split(",")]
        assert len(args) == len(declared)
        for a, d in zip(args[2:], declared[2:]):
            assert d == (a.removeprefix("fort_handle_") + "_handle" if a.startswith("fort_handle_") else a)


def _write_app(tmp_path, minimum=1, extra=""):
    (tmp_path / "src").mkdir()
    (tmp_path / "src" / "kernels.f90").write_text(SYNTHETIC)
    (tmp_path / "src" / "main.f90").write_text(
        "program main\n  use MomentumAdvection\n  implicit none\n  ! timed\n  call work()\nend program main\n")
    (tmp_path / "app.toml").write_text(f"""
name = "Synthetic"
sources = ["src/kernels.f90", "src/main.f90"]
program = "src/main.f90"
[variants.default]
defines = ["SMALL"]
[[selection]]
label = "advection"
procedures = ["momentumadvection::*"]
minimum_nests = {minimum}
[[edit]]
file = "main.f90"
at = "  ! timed\\n"
action = "before"
text = "  !$fort enter\\n"
[[edit]]
file = "main.f90"
at = "end program main"
action = "before"
text = "  !$fort close\\n"
[build]
fortran_options = ["-O2"]
[[executable]]
name = "synthetic"
library = "resident"
[[executable]]
name = "synthetic-native"
library = "native"
{extra}""")
    return tmp_path / "app.toml"


def test_described_application_prepares_resident_and_native_trees(tmp_path):
    app = application.load(_write_app(tmp_path))
    application.prepare(app, tmp_path / "out")
    out = tmp_path / "out"
    assert (out / "native" / "kernels.f90").read_text() == SYNTHETIC
    resident_main = (out / "resident" / "main.f90").read_text()
    assert resident_main.index("begin_epoch") < resident_main.index("! timed")
    assert resident_main.index("call resident%close()") < resident_main.index("end program main")
    _balanced(resident_main)
    cmake = (out / "CMakeLists.txt").read_text()
    assert "project(Synthetic LANGUAGES Fortran)" in cmake
    assert "-ffp-contract=off" in cmake and "-DSMALL" in cmake
    assert 'add_executable(synthetic "resident/main.f90")' in cmake
    assert 'add_executable(synthetic-native "native/main.f90")' in cmake
    assert "fort_resident_domain.f90" in cmake and "fort_shared_entries.f90" in cmake
    report = json.loads((out / "resident_build.json").read_text())
    assert report["nests"] == {"advection": 1}
    assert [d["directive"] for d in report["directives"]] == ["enter", "close"]


def test_minimum_nests_is_enforced(tmp_path):
    app = application.load(_write_app(tmp_path, minimum=2))
    with pytest.raises(application.DescriptionError, match="fewer than minimum_nests = 2"):
        application.prepare(app, tmp_path / "out")


@pytest.mark.parametrize("extra, message", [
    ("[[patch]]\nfile = 'x'\n", "outside the advection path"),
    ("[unexpected]\nx = 1\n", "unknown keys"),
    ("[[edit]]\nfile = 'main.f90'\nat = 'nowhere'\naction = 'before'\ntext = 'x'\n", "anchor found 0 times"),
    ("[[edit]]\nfile = 'main.f90'\nat = 'x'\naction = 'sideways'\ntext = 'x'\n", "before, after or replace"),
])
def test_description_errors(tmp_path, extra, message):
    path = _write_app(tmp_path, extra=extra)
    with pytest.raises(application.DescriptionError, match=message):
        application.prepare(application.load(path), tmp_path / "out")


def test_cli_prepare_only(tmp_path, capsys):
    assert cli.main([str(_write_app(tmp_path)), "--output", str(tmp_path / "out"), "--prepare-only"]) == 0
    line = json.loads(capsys.readouterr().out)
    assert line == {"application": "Synthetic", "entries": 1, "nests": {"advection": 1}, "directives": 2,
                    "outcome": "prepared"}
    (tmp_path / "bad").mkdir()
    assert cli.main([str(_write_app(tmp_path / "bad", minimum=5)), "--output", str(tmp_path / "o2")]) == 1


def test_cli_takes_the_reference_command_line(tmp_path, capsys):
    app = str(_write_app(tmp_path))
    out = str(tmp_path / "out")
    # the reference's full argument list, preparing only
    assert cli.main([app, "--output", out, "--fortran", "gfortran", "--cxx", "g++", "--architecture", "103a",
                     "--jobs", "2", "--prepare-only"]) == 0
    capsys.readouterr()
    # building what was prepared: no Fortran compiler here, so it stops after the preparation it finds
    assert cli.main([app, "--output", out, "--build-prepared"]) == 0
    assert json.loads(capsys.readouterr().out)["application"] == "Synthetic"
    for extra, message in ((["--architecture", "86"], "built for sm_103a"),
                           (["--input", "elmm=/tmp"], "outside the advection path"),
                           (["--prepare-only", "--build-prepared"], "choose preparation")):
        assert cli.main([app, "--output", out, *extra]) == 1
        assert message in capsys.readouterr().err


@pytest.mark.skipif(not CDU_TOML.exists(), reason="the reference's cdu benchmark is not on this machine")
def test_reference_cdu_description_prepares(tmp_path):
    app = application.load(CDU_TOML)
    application.prepare(app, tmp_path)
    report = app.report
    spliced = {e["procedure"]: e["entry"] for e in report["entries"]}
    for name in ("set", "multiply", "cdudiv", "cduadv", "cdu"):
        assert spliced[f"momentumadvection::{name}"] == emission.entry_for(f"MomentumAdvection::{name}").symbol
    assert report["nests"]["advection"] >= 4
    main = (tmp_path / "resident" / "main.f90").read_text()
    assert main.index("begin_epoch") < main.index("! ---- warm-up ----")
    assert main.index("end_epoch") < main.index("call system_clock(t_end)")
    assert main.index("call resident%close()") < main.index("deallocate(U, V, W, U2)")
    # host statements on the fields: the initialisation is handed over, the checksum observed, the
    # deallocation released
    assert [(b["block"], b["arrays"]) for b in report["host_blocks"]] == [
        ("hand-over", ["u", "u2", "v", "w"]), ("observe", ["u2"]), ("release", ["u", "u2", "v", "w"])]
    kernels = (tmp_path / "resident" / "cdu.f90").read_text()
    _balanced(kernels)
    _balanced(main)
    assert (tmp_path / "native" / "cdu.f90").read_text() == (CDU_TOML.parent / "src" / "cdu.f90").read_text()


def test_fortran_modules_bind_only_declared_c_entry_points():
    """Every bind(C) name the Fortran modules call is declared by the C ABI headers."""
    root = Path(emission.__file__).parents[2]
    headers = "".join(p.read_text() for p in (root.parent / "include").glob("*.h"))
    for source in (root / "fortran").glob("*.f90"):
        for name in re.findall(r"bind\(C,\s*name='(\w+)'\)", source.read_text()):
            assert re.search(rf"\b{name}\s*\(", headers), f"{source.name}: {name} is not in include/*.h"


EDIT_SOURCE = """module m
contains
  subroutine first(a)
    real :: a
    call helper(a)
    a = a + 1
  end subroutine first

  subroutine second(a)
    real :: a
    a = a + 1
  end subroutine second
end module m
"""


def _edited(**fields):
    return application.apply_edit(EDIT_SOURCE, application.Edit(file="m.f90", **fields))


def test_edits_locate_by_anchor_call_span_procedure_and_module_end():
    """The reference's edit locators (compiler/resident/application.py:49-57; its tests in
    test_resident_application_description.py:40-60): an anchor confined to a procedure, a CALL statement from the
    start of its line, a span between two texts, a whole procedure, and the end of a module."""
    text = _edited(procedure="second", at="    a = a + 1\n", action="after", text="    a = 2 * a\n")
    assert "    a = a + 1\n    a = 2 * a\n  end subroutine second" in text
    with pytest.raises(application.DescriptionError, match="expected one"):
        _edited(at="    a = a + 1\n", action="after", text="x")
    text = _edited(procedure="first", call="helper", action="replace", text="    if (on) then\n{original}\n    end if")
    assert "    if (on) then\n    call helper(a)\n    end if\n" in text
    text = _edited(procedure="first", between=["call helper", "a = a + 1"], action="replace", text="! gone")
    assert "    ! gone\n  end subroutine first" in text
    text = _edited(procedure="second", action="before", text="  subroutine third\n  end subroutine third\n\n")
    assert text.index("subroutine third") < text.index("subroutine second(a)")
    text = _edited(module_end="m", action="before", text="\n  ! last\n")
    assert text.endswith("  end subroutine second\n\n  ! last\nend module m\n")


@pytest.mark.parametrize("edit, message", [
    ("[[edit]]\nfile = 'main.f90'\naction = 'after'\ntext = ''\n", "locates no place"),
    ("[[edit]]\nfile = 'main.f90'\nat = 'x'\naction = 'after'\ntext = ''\nfloor = 3\n", "unknown keys in edit"),
    ("[[edit]]\nfile = 'main.f90'\nbetween = ['a']\naction = 'replace'\ntext = ''\n", "two pieces of text"),
])
def test_edits_are_checked_where_the_description_is_read(tmp_path, edit, message):
    with pytest.raises(application.DescriptionError, match=message):
        application.load(_write_app(tmp_path, extra=edit))


def test_cli_fast_fp_drops_the_strict_option_and_sets_the_contract(tmp_path, capsys):
    """--fast-fp (the reference's option, compiler/resident/__main__.py:34-35): both builds drop
    -ffp-contract=off (compiler/resident/build.py:57-66) and the resident objects are preprocessed with
    F2C_FAST_FP, under which the residency domain opens its contexts in the fast-fp numerical contract."""
    app = str(_write_app(tmp_path))
    strict, fast = tmp_path / "strict", tmp_path / "fast"
    assert cli.main([app, "--output", str(strict), "--prepare-only"]) == 0
    assert cli.main([app, "--output", str(fast), "--prepare-only", "--fast-fp"]) == 0
    capsys.readouterr()
    strict_cmake, fast_cmake = (strict / "CMakeLists.txt").read_text(), (fast / "CMakeLists.txt").read_text()
    assert "-ffp-contract=off" in strict_cmake and "-ffp-contract=off" not in fast_cmake
    assert "F2C_FAST_FP" not in strict_cmake
    assert "target_compile_definitions(resident_objects PRIVATE F2C_FAST_FP)" in fast_cmake
    assert json.loads((fast / "resident_build.json").read_text())["numerics"] == "fast"
    assert json.loads((strict / "resident_build.json").read_text())["numerics"] == "strict"
    domain = (Path(emission.PACKAGE_ROOT) / "fortran" / "fort_resident_domain.f90").read_text()
    block = domain[domain.index("#ifdef F2C_FAST_FP"):domain.index("#endif")]
    assert "fort_scope_numerics_set_v1(self%context, FORT_SCOPE_NUMERICS_FAST)" in block
