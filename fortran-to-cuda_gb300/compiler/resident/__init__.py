"""The resident build surface: the domain object, the ``!$fort`` directives, the call block and the description.

``domain.ResidentDomain`` is the Python counterpart of the Fortran residency
object (compiler/runtime/resident_domain.f90 of the reference), for drivers
written in Python and for tests that act like a spliced Fortran program.
"""
