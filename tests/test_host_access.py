"""Host-access blocks: host statements that touch arrays the entries keep on the device.

The reference wraps such statements while it splices
(compiler/scopes/resident_splice.py:209-300): reads are observed, writes are
handed to the host and back, deallocations release first, statements that
control can leave publish everything, and a loop condition evaluated between
entry calls ends the epoch. No Fortran compiler exists here, so the tests read
the generated text: which statements got which block, with which arrays, and
that every block is closed.
"""

import re

import pytest

from compiler import emission
from compiler.resident import application, host_access, splice

KERNELS = """\
module MomentumAdvection
  implicit none
contains
  subroutine CDU(U2, U, V, W, dxmin, dymin, dzmin, Unx, Uny, Unz)
    real(8), intent(inout) :: U2(:,:,:)
    real(8), intent(in) :: U(:,:,:), V(:,:,:), W(:,:,:)
    real(8), intent(in) :: dxmin, dymin, dzmin
    integer, intent(in) :: Unx, Uny, Unz
    U2 = 0
  end subroutine CDU
end module MomentumAdvection
"""

MAIN = """\
module stepping
  use MomentumAdvection
  implicit none
  real(8), allocatable :: shared(:,:,:)
contains
  subroutine advance(A, B, C, D, n)
    real(8), intent(inout) :: A(:,:,:)
    real(8), intent(in) :: B(:,:,:), C(:,:,:), D(:,:,:)
    integer, intent(in) :: n
    call CDU(A, B, C, D, 1d0, 1d0, 1d0, n, n, n)
    A = 0.5d0 * A
  end subroutine advance
  subroutine report(X)
    real(8), intent(in) :: X(:,:,:)
    print *, sum(X)
  end subroutine report
  subroutine smooth(X)
    real(8), intent(inout) :: X(:,:,:)
    X = 0.9d0 * X
  end subroutine smooth
end module stepping

program main
  use stepping
  implicit none
  real(8), allocatable :: U(:,:,:), V(:,:,:), W(:,:,:), U2(:,:,:), tmp(:,:,:)
  real(8) :: s
  integer :: it, n
  n = 8
  allocate(U(n+2,n+2,n+2), V(n+2,n+2,n+2), W(n+2,n+2,n+2), U2(n+2,n+2,n+2))
  call random_number(U)
  !$fort enter
  do it = 1, 10
    call CDU(U2, U, V, W, 1d0, 1d0, 1d0, n, n, n)
    U = U + 0.1d0 * U2
    s = sum(U2)
    if (s > 1d9) print *, 'large', maxval(V)
    if (s < 0) then
      U2 = 0
      exit
    end if
  end do
  do while (maxval(U2) > 1d0)
    call CDU(U2, U, V, W, 1d0, 1d0, 1d0, n, n, n)
  end do
  if (sum(W) > 0) then
    call advance(U2, U, V, W, n)
  end if
  call smooth(V)
  call report(W)
  do it = 1, n
    if (U(1,1,it) < 0) exit
    U(1,1,it) = 1
  end do
  !$fort leave
  print *, 'checksum', sum(U2(2:n+1,2:n+1,2:n+1))
  n = 0
  deallocate(U2)
  deallocate(U, V, W)
end program main
"""


def _wrap(files):
    spliced, entries, texts = set(), {}, {}
    for name, text in files.items():
        out, done = splice.splice(text, ["momentumadvection::cdu"])
        texts[name] = out
        for d in done:
            spliced.add(d.procedure)
            entry = emission.entry_for(d.procedure)
            entries[d.procedure.split("::")[-1]] = [(n, p.name.lower()) for n, p in enumerate(entry.params)
                                                    if p.kind == "array"]
    return host_access.wrap(texts, entries, spliced)


def _balanced(text):
    blocks = sum(1 for ln in text.splitlines() if ln.split("!")[0].strip().lower() == "block")
    ends = sum(1 for ln in text.splitlines() if ln.split("!")[0].strip().lower() == "end block")
    ifs = sum(1 for ln in text.splitlines() if re.match(r"\s*if\s*\(.*\)\s*then\s*$", ln.split("!")[0], re.I))
    endifs = sum(1 for ln in text.splitlines() if ln.split("!")[0].strip().lower() in ("endif", "end if"))
    assert (blocks, ifs) == (ends, endifs)


@pytest.fixture(scope="module")
def wrapped():
    files, records = _wrap({"kernels.f90": KERNELS, "main.f90": MAIN})
    return files, {(r["file"], r["line"]): r for r in records}


def _line(text, statement, nth=0):
    lines = MAIN.splitlines()
    hits = [n + 1 for n, ln in enumerate(lines) if ln.strip() == statement]
    return hits[nth]


def test_reads_writes_and_releases_get_their_blocks(wrapped):
    files, records = wrapped
    main = files["main.f90"]
    _balanced(main)
    got = {(r["block"], tuple(r["arrays"])): line for (f, line), r in records.items() if f == "main.f90"}
    line = lambda s, n=0: _line(MAIN, s, n)
    # random_number writes U: handed to the host and back (outside an epoch the block only tests active)
    assert got[("hand-over", ("u",))] == line("call random_number(U)")
    # U = U + 0.1*U2 reads U2 and writes U; s = sum(U2) reads U2: one span of two statements
    assert records[("main.f90", line("U = U + 0.1d0 * U2"))]["arrays"] == ["u", "u2"]
    # the one-line IF whose condition names no array: the access sits inside the IF
    assert records[("main.f90", line("if (s > 1d9) print *, 'large', maxval(V)"))]["block"] == "observe"
    assert "if (s > 1d9) then" in main and "  print *, 'large', maxval(V)\n" in main
    # a loop condition evaluated between entry calls ends the epoch
    assert records[("main.f90", line("do while (maxval(U2) > 1d0)"))]["block"] == "leave"
    # an IF condition evaluated once before an entry path is observed before the construct
    assert records[("main.f90", line("if (sum(W) > 0) then"))] == {
        "file": "main.f90", "line": line("if (sum(W) > 0) then"), "block": "observe", "arrays": ["w"]}
    # the callee's dummy decides: intent(inout) hands over, intent(in) observes
    assert records[("main.f90", line("call smooth(V)"))]["block"] == "hand-over"
    # smooth, report and the loop after them are one span; the loop's EXIT stays inside the span
    assert records[("main.f90", line("call smooth(V)"))]["arrays"] == ["u", "v", "w"]
    assert ("main.f90", line("do it = 1, n")) not in records
    # statements that control leaves (EXIT of the enclosing loop) while they write U2 publish everything first
    assert records[("main.f90", line("if (s < 0) then"))]["block"] == "publish"
    # the checksum after the epoch reads U2; the deallocations release (after observing what is read)
    assert records[("main.f90", line("print *, 'checksum', sum(U2(2:n+1,2:n+1,2:n+1))"))]["block"] == "observe"
    assert records[("main.f90", line("deallocate(U2)"))] == {
        "file": "main.f90", "line": line("deallocate(U2)"), "block": "release", "arrays": ["u", "u2", "v", "w"]}
    tail = main[main.index("deallocate(U2)") - 600:]
    assert "if (allocated(u2)) call resident%release_real(u2)" in tail


def test_entry_calls_and_unbound_statements_are_left_alone(wrapped):
    files, records = wrapped
    main = files["main.f90"].splitlines()
    lines = MAIN.splitlines()
    for statement in ("n = 8", "call CDU(U2, U, V, W, 1d0, 1d0, 1d0, n, n, n)"):
        at = [n + 1 for n, ln in enumerate(lines) if ln.strip() == statement]
        assert all(("main.f90", a) not in records for a in at)
    # no block in the spliced kernel module
    assert not [r for r in records.values() if r["file"] == "kernels.f90"]
    # allocate names no array that is already held
    assert ("main.f90", _line(MAIN, "allocate(U(n+2,n+2,n+2), V(n+2,n+2,n+2), W(n+2,n+2,n+2), U2(n+2,n+2,n+2))")) \
        not in records
    assert sum(1 for ln in main if "call CDU(" in ln) == sum(1 for ln in lines if "call CDU(" in ln) == 3


def test_bindings_flow_through_procedures_that_reach_entries(wrapped):
    files, records = wrapped
    # advance() passes its dummy A to CDU and then scales it on the host: A is bound inside advance
    stepping = files["main.f90"]
    at = _line(MAIN, "A = 0.5d0 * A")
    assert records[("main.f90", at)]["block"] == "hand-over"
    assert records[("main.f90", at)]["arrays"] == ["a"]
    # the call of advance() is an entry path: no block around it
    assert ("main.f90", _line(MAIN, "call advance(U2, U, V, W, n)")) not in records
    # smooth() binds nothing itself (it reaches no entry): its statement is not wrapped inside it
    assert ("main.f90", _line(MAIN, "X = 0.9d0 * X")) not in records
    assert "fort_held(1) = resident%held(a)" in stepping


def test_block_text_asks_the_domain_and_guards_allocatables(wrapped):
    files, _ = wrapped
    main = files["main.f90"]
    start = main.index("block", main.index("n = 8"))
    block = main[start:main.index("end block", start)]
    assert "use fort_resident_application, only: resident" in block
    assert "fort_host = resident%active" in block
    assert "if (allocated(u)) fort_held(1) = resident%held(u)" in block
    assert "call resident%host_modify(fort_held)" in block
    after = main[main.index("call random_number(U)"):]
    assert after.index("if (fort_host) call resident%host_done(fort_held)") < after.index("end block")


def test_a_branch_target_that_touches_device_arrays_is_refused():
    text = MAIN.replace("  call smooth(V)\n", "  go to 20\n20 call smooth(V)\n")
    with pytest.raises(host_access.HostAccessError, match="branch target"):
        _wrap({"kernels.f90": KERNELS, "main.f90": text})


def test_internal_procedures_see_their_hosts_bindings():
    text = MAIN.replace("end program main", "contains\n  subroutine zero()\n    U2 = 0\n  end subroutine zero\n"
                                            "end program main")
    files, records = _wrap({"kernels.f90": KERNELS, "main.f90": text})
    at = text.splitlines().index("    U2 = 0") + 1
    assert records and [r for r in records if r["line"] == at and r["arrays"] == ["u2"]]
    _balanced(files["main.f90"])


def test_prepare_reports_host_blocks(tmp_path):
    (tmp_path / "src").mkdir()
    (tmp_path / "src" / "kernels.f90").write_text(KERNELS)
    (tmp_path / "src" / "main.f90").write_text(MAIN)
    (tmp_path / "app.toml").write_text("""
name = "HostAccess"
sources = ["src/kernels.f90", "src/main.f90"]
program = "src/main.f90"
[[selection]]
label = "advection"
procedures = ["momentumadvection::cdu"]
[[executable]]
name = "host-access"
library = "resident"
""")
    app = application.prepare(application.load(tmp_path / "app.toml"), tmp_path / "out")
    blocks = app.report["host_blocks"]
    assert {b["block"] for b in blocks} >= {"hand-over", "observe", "leave", "publish", "release"}
    resident = (tmp_path / "out" / "resident" / "main.f90").read_text()
    assert "!$fort" not in resident and "call resident%begin_epoch" in resident
    _balanced(resident)
    # the directives' own expansions are not wrapped again
    assert resident.count("call resident%end_epoch()") == 2     # the leave directive and the do-while block


def test_labelled_loops_and_select_constructs():
    """An old-style labelled DO is one construct up to its terminal statement; SELECT CASE around an entry call
    is entered and each CASE body gets its own blocks."""
    text = MAIN.replace("  call smooth(V)\n", """  do 30 it = 1, n
    U(1,1,it) = 2
30 continue
  select case (n)
  case (1)
    call CDU(U2, U, V, W, 1d0, 1d0, 1d0, n, n, n)
  case default
    V = 0
  end select
  call smooth(V)
""")
    files, records = _wrap({"kernels.f90": KERNELS, "main.f90": text})
    lines = text.splitlines()
    at = {r["line"]: r for r in records}
    loop = lines.index("  do 30 it = 1, n") + 1
    assert at[loop]["block"] == "hand-over" and at[loop]["arrays"] == ["u"]
    assert lines.index("  select case (n)") + 1 not in at         # the selector names no array
    assert at[lines.index("    V = 0") + 1]["arrays"] == ["v"]    # inside CASE DEFAULT
    out = files["main.f90"]
    _balanced(out)
    # the labelled terminal stays inside the block around its loop
    wrapped = out[out.index("do 30 it = 1, n"):]
    assert wrapped.index("30 continue") < wrapped.index("call resident%host_done")
