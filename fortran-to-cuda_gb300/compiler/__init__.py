"""GB300-native host of the resident advection path.

Mirrors the reference's ``compiler`` package where the hot path touches it:
``compiler.runtime`` (the native residency runtime and its ABI),
``compiler.emission`` (thin C-ABI entries into hand-written sm_103a templates),
``compiler.scheduling`` (tile and z-block autotuner) and ``compiler.resident``
(the TOML description, ``!$fort`` directives and the splice call block).
"""

__all__ = ["native"]
