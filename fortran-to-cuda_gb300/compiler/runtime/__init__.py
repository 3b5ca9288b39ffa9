"""The residency runtime: ctypes bindings of the fort_scope_* ABI (include/scoped_runtime.h).

``abi.bind(library)`` declares every entry point on a loaded library: the
product library (CUDA backend) or the CPU test build of the same runtime.
"""
