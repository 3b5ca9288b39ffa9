"""Entry emission and the exported C ABI (CPU only: no GPU call is made)."""

import re
import subprocess

import numpy as np
import pytest

from compiler import emission, native
from compiler.resident.domain import ResidentDomain
from compiler.runtime import abi


def test_generated_files_are_current_and_deterministic():
    first = emission.outputs()
    second = emission.outputs()
    assert first == second
    for path, text in first.items():
        assert path.read_text() == text, f"{path} is stale: regenerate with compiler.emission.write_entries()"


def test_entry_names_follow_the_reference_scheme():
    seen = set()
    for e in emission.registry():
        assert re.fullmatch(r"cpp_fort_shared_[0-9a-f]{12}", e.symbol)
        assert e.fortran_module == "fort_shared_" + e.symbol[-12:]
        assert e.symbol not in seen
        seen.add(e.symbol)
    cdu = emission.entry_for("MomentumAdvection::CDU")
    assert [p.name for p in cdu.params] == ["U2", "U", "V", "W", "dxmin", "dymin", "dzmin", "Unx", "Uny", "Unz"]
    assert [p.intent for p in cdu.arrays()] == ["out", "in", "in", "in"]


def _exports(path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True, check=True)
    return {line.split()[-1] for line in out.stdout.splitlines() if line.split()}


def _declared(header):
    text = header.read_text()
    pattern = r"^(?:[A-Za-z_][A-Za-z0-9_]*\s+\**)+((?:fort_scope|cpp_fort_shared|f2c)_[A-Za-z0-9_]+)\("
    return set(re.findall(pattern, text, flags=re.MULTILINE))


def test_library_exports_every_declared_symbol():
    lib = native.build()
    exported = _exports(lib)
    root = native.INCLUDE
    declared = set()
    for header in ("scoped_runtime.h", "fort_shared_entries.h", "f2c_advection.h"):
        declared |= _declared(root / header)
    missing = sorted(declared - exported)
    assert not missing, missing
    assert len([s for s in declared if s.startswith("cpp_fort_shared_")]) == len(emission.registry())


def test_fortran_bindings_link_against_exported_names():
    exported = _exports(native.build())
    text = emission.FORTRAN_INTERFACES.read_text()
    for name in re.findall(r"bind\(C, name='([a-z0-9_]+)'\)", text):
        assert name in exported


def test_entries_decline_without_a_gpu_and_touch_nothing():
    """On a machine without a device an entry cannot reserve storage: it declines and nothing changes."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("this checks the behaviour without a device")
    lib = native.runtime()
    dom = ResidentDomain(lib)
    fns = emission.bind(lib)
    dom.begin_epoch(budget=1 << 30)
    arrays = [np.full((6, 6, 6), float(n)) for n in range(4)]
    hs = [dom.bind_real64(a) for a in arrays]
    for mode in (abi.NATIVE, abi.GPU):
        status = emission.call(fns, "momentumadvection::cdu", dom.context, mode, hs, [1.0, 1.0, 1.0], [4, 4, 4])
        assert status == abi.DECLINED
    dom.end_epoch()
    dom.close()
    for n, a in enumerate(arrays):
        assert (a == n).all()
