"""Thin emitter of C-ABI numerical entries into the hand-written sm_103a templates."""


def write_entries() -> None:
    """Write the generated entry sources into csrc/entries (none are registered yet)."""
    return None
