! Fortran binding of the GB300 residency runtime (include/scoped_runtime.h).
!
! Public names, constants and record layouts are those the spliced code of a
! resident build uses (module fort_scoped_memory of the reference,
! compiler/runtime/scoped_memory.f90), so generated call blocks and the
! residency domain compile unchanged against this library. Only the part of
! the interface the advection path uses is bound here.
module fort_scoped_memory
  use, intrinsic :: iso_c_binding
  implicit none
  private

  integer(c_int), parameter, public :: FORT_SCOPE_OK = 0, FORT_SCOPE_ARGUMENT = 1, FORT_SCOPE_STALE = 2, &
    FORT_SCOPE_ALIAS = 3, FORT_SCOPE_RESOURCE = 4, FORT_SCOPE_BOUNDARY = 5, FORT_SCOPE_EXECUTION = 6, &
    FORT_SCOPE_UNINITIALIZED = 7, FORT_SCOPE_STATE = 8, FORT_SCOPE_DECLINED = 9
  integer(c_int), parameter, public :: FORT_SCOPE_BYTES = 0, FORT_SCOPE_REAL32 = 1, FORT_SCOPE_REAL64 = 2, &
    FORT_SCOPE_INTEGER32 = 3, FORT_SCOPE_LOGICAL = 4
  integer(c_int), parameter, public :: FORT_SCOPE_READ_ALL = 1, FORT_SCOPE_WRITE_ALL = 2, FORT_SCOPE_OVERWRITE_ALL = 4
  integer(c_int), parameter, public :: FORT_SCOPE_NATIVE = 0, FORT_SCOPE_GPU = 1

  type, bind(C), public :: fort_scope_section
    type(c_ptr) :: lower = c_null_ptr
    type(c_ptr) :: upper = c_null_ptr
  end type

  type, bind(C), public :: fort_scope_access
    integer(c_int32_t) :: flags = 0
    integer(c_size_t) :: read_count = 0
    type(c_ptr) :: reads = c_null_ptr
    integer(c_size_t) :: write_count = 0
    type(c_ptr) :: writes = c_null_ptr
    integer(c_size_t) :: overwrite_count = 0
    type(c_ptr) :: overwrites = c_null_ptr
  end type

  type, bind(C), public :: fort_scope_layout
    integer(c_int32_t) :: rank = 0, element_type = 0
    integer(c_size_t) :: element_bytes = 0
    type(c_ptr) :: host = c_null_ptr
    type(c_ptr) :: extents = c_null_ptr
    type(c_ptr) :: lower_bounds = c_null_ptr
    integer(c_int64_t) :: generation = 0
  end type

  type, bind(C), public :: fort_scope_stats
    integer(c_int64_t) :: uploads = 0, downloads = 0, upload_bytes = 0, download_bytes = 0
    integer(c_int64_t) :: allocations = 0, allocated_bytes = 0, peak_device_bytes = 0
    integer(c_int64_t) :: launches = 0, waits = 0, reconciliations = 0
  end type

  public :: fort_scope_abi_version, fort_scope_error, fort_scope_device_budget_default_v1, &
    fort_scope_domain_create_v1, fort_scope_create_in_domain_v1, fort_scope_set_device_budget, &
    fort_scope_domain_budget_get_v1, fort_scope_register, fort_scope_layout_get, fort_scope_observe_v1, &
    fort_scope_host_begin, fort_scope_host_end, fort_scope_unregister, fort_scope_retire_v1, fort_scope_close, &
    fort_scope_domain_close_v1, fort_scope_wait, fort_scope_stats_get, fort_scope_forget_definition

  interface
    function fort_scope_abi_version() bind(C, name='fort_scope_abi_version') result(version)
      import :: c_int32_t
      integer(c_int32_t) :: version
    end function

    function fort_scope_error() bind(C, name='fort_scope_error') result(message)
      import :: c_ptr
      type(c_ptr) :: message
    end function

    function fort_scope_device_budget_default_v1(device, bytes) bind(C, name='fort_scope_device_budget_default_v1') &
        result(status)
      import :: c_int, c_size_t
      integer(c_int), value :: device
      integer(c_size_t), intent(out) :: bytes
      integer(c_int) :: status
    end function

    function fort_scope_domain_create_v1(device, domain) bind(C, name='fort_scope_domain_create_v1') result(status)
      import :: c_int, c_int64_t
      integer(c_int), value :: device
      integer(c_int64_t), intent(out) :: domain
      integer(c_int) :: status
    end function

    function fort_scope_create_in_domain_v1(domain, context) bind(C, name='fort_scope_create_in_domain_v1') &
        result(status)
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: domain
      integer(c_int64_t), intent(out) :: context
      integer(c_int) :: status
    end function

    function fort_scope_set_device_budget(context, bytes) bind(C, name='fort_scope_set_device_budget') result(status)
      import :: c_int, c_int64_t, c_size_t
      integer(c_int64_t), value :: context
      integer(c_size_t), value :: bytes
      integer(c_int) :: status
    end function

    function fort_scope_domain_budget_get_v1(domain, budget, unclaimed) bind(C, name='fort_scope_domain_budget_get_v1') &
        result(status)
      import :: c_int, c_int64_t, c_size_t
      integer(c_int64_t), value :: domain
      integer(c_size_t), intent(out) :: budget, unclaimed
      integer(c_int) :: status
    end function

    function fort_scope_register(context, identity, generation, layout, host_initialized, buffer) &
        bind(C, name='fort_scope_register') result(status)
      import :: c_int, c_int64_t, fort_scope_layout
      integer(c_int64_t), value :: context, identity, generation
      type(fort_scope_layout), intent(in) :: layout
      integer(c_int), value :: host_initialized
      integer(c_int64_t), intent(out) :: buffer
      integer(c_int) :: status
    end function

    function fort_scope_layout_get(context, buffer, layout) bind(C, name='fort_scope_layout_get') result(status)
      import :: c_int, c_int64_t, fort_scope_layout
      integer(c_int64_t), value :: context, buffer
      type(fort_scope_layout), intent(out) :: layout
      integer(c_int) :: status
    end function

    function fort_scope_forget_definition(context, buffer) bind(C, name='fort_scope_forget_definition') result(status)
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: context, buffer
      integer(c_int) :: status
    end function

    function fort_scope_observe_v1(context, buffers, count) bind(C, name='fort_scope_observe_v1') result(status)
      import :: c_int, c_int64_t, c_ptr, c_size_t
      integer(c_int64_t), value :: context
      type(c_ptr), value :: buffers
      integer(c_size_t), value :: count
      integer(c_int) :: status
    end function

    function fort_scope_host_begin(context, buffer, access) bind(C, name='fort_scope_host_begin') result(status)
      import :: c_int, c_int64_t, fort_scope_access
      integer(c_int64_t), value :: context, buffer
      type(fort_scope_access), intent(in) :: access
      integer(c_int) :: status
    end function

    function fort_scope_host_end(context, buffer) bind(C, name='fort_scope_host_end') result(status)
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: context, buffer
      integer(c_int) :: status
    end function

    function fort_scope_unregister(context, buffer) bind(C, name='fort_scope_unregister') result(status)
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: context, buffer
      integer(c_int) :: status
    end function

    function fort_scope_retire_v1(context, buffer) bind(C, name='fort_scope_retire_v1') result(status)
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: context, buffer
      integer(c_int) :: status
    end function

    function fort_scope_close(context) bind(C, name='fort_scope_close') result(status)
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: context
      integer(c_int) :: status
    end function

    function fort_scope_domain_close_v1(domain) bind(C, name='fort_scope_domain_close_v1') result(status)
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: domain
      integer(c_int) :: status
    end function

    function fort_scope_wait(context) bind(C, name='fort_scope_wait') result(status)
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: context
      integer(c_int) :: status
    end function

    function fort_scope_stats_get(context, stats) bind(C, name='fort_scope_stats_get') result(status)
      import :: c_int, c_int64_t, fort_scope_stats
      integer(c_int64_t), value :: context
      type(fort_scope_stats), intent(out) :: stats
      integer(c_int) :: status
    end function
  end interface
end module fort_scoped_memory
