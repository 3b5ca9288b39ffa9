! The residency domain a resident build's directives and call blocks use.
!
! Public names and behaviour are those the spliced code relies on (module
! fort_resident_domain of the reference, compiler/runtime/resident_domain.f90):
! begin_epoch creates the domain and its context on first use (default budget
! from the runtime, or the caller's) and advances the generation; bind_real64
! registers an array by the address of its first element and its extents and
! returns the handle already held for that storage within the epoch (a
! tolerant binding answers 0 for an empty or non-contiguous array); observe
! publishes named arrays; publish observes and unregisters every non-persistent
! array; end_epoch publishes and ends the epoch; close releases the context and
! the domain. held answers the handle of the storage an array lies in (0 when
! the domain keeps none); host_modify hands arrays to host code that may change
! them and host_done hands them back. observe_field takes the address of one
! field in the first element of an array of derived type; this domain keeps no
! such field on the device, so the field is already current on the host and
! nothing moves. resident_require stops the program on a
! nonzero status: work that failed after it started is never replayed.
module fort_resident_domain
  use, intrinsic :: iso_c_binding
  use, intrinsic :: iso_fortran_env, only: error_unit
  use fort_scoped_memory
  implicit none
  private
  public :: resident_domain, resident_require

  type :: held_storage
    integer(c_int64_t) :: identity = 0, handle = 0
    integer(c_size_t), allocatable :: extents(:)
    integer(c_int64_t), allocatable :: lower(:)
    logical :: persistent = .false.
  end type

  type :: resident_domain
    integer(c_int64_t) :: domain = 0, context = 0, generation = 0
    integer(c_int64_t) :: stamp = 0
    logical :: active = .false.
    type(held_storage), allocatable, private :: storage(:)
  contains
    procedure :: begin_epoch
    procedure :: unclaimed
    procedure :: bind_real64
    generic :: bind => bind_real64
    procedure :: held
    procedure :: host_modify
    procedure :: host_done
    procedure :: release
    procedure :: observe
    procedure :: observe_field
    procedure :: publish
    procedure :: end_epoch
    procedure :: close
  end type

contains

  subroutine resident_require(status)
    integer(c_int), intent(in) :: status
    character(kind=c_char), pointer :: text(:)
    integer :: length
    if (status == FORT_SCOPE_OK) return
    write(error_unit, '(a,i0,a)') 'Resident runtime failed (status ', status, '); source work will not be replayed.'
    if (c_associated(fort_scope_error())) then
      call c_f_pointer(fort_scope_error(), text, [512])
      length = 0
      do while (length < 511)
        if (text(length + 1) == c_null_char) exit
        length = length + 1
      enddo
      if (length > 0) write(error_unit, '(a,512a1)') 'Runtime: ', text(:length)
    endif
    error stop 'resident execution failure'
  end subroutine

  subroutine begin_epoch(self, device, budget)
    class(resident_domain), intent(inout) :: self
    integer(c_int), intent(in) :: device
    integer(c_size_t), optional, intent(in) :: budget
    integer(c_size_t) :: bytes
    if (self%active) error stop 'nested storage epoch'
    if (self%domain == 0) then
      if (present(budget)) then
        bytes = budget
      else
        call resident_require(fort_scope_device_budget_default_v1(device, bytes))
      endif
      call resident_require(fort_scope_domain_create_v1(device, self%domain))
      call resident_require(fort_scope_create_in_domain_v1(self%domain, self%context))
      call resident_require(fort_scope_set_device_budget(self%context, bytes))
      allocate(self%storage(0))
    endif
    self%generation = self%generation + 1
    self%active = .true.
  end subroutine

  function unclaimed(self) result(bytes)
    class(resident_domain), intent(in) :: self
    integer(c_size_t) :: bytes, budget
    call resident_require(fort_scope_domain_budget_get_v1(self%domain, budget, bytes))
  end function

  function bind_real64(self, values, lower, initialized, persistent, origin, tolerant) result(handle)
    class(resident_domain), intent(inout) :: self
    real(c_double), target, intent(in) :: values(..)
    integer, intent(in) :: lower(:)
    logical, intent(in) :: initialized
    logical, optional, intent(in) :: persistent, tolerant
    character(*), optional, intent(in) :: origin
    integer(c_int64_t) :: handle
    integer(c_size_t), allocatable, target :: extents(:)
    integer(c_int64_t), allocatable, target :: bounds(:)
    type(fort_scope_layout) :: layout
    type(held_storage) :: item
    integer(c_int64_t) :: identity, generation
    logical :: keep, forgiving
    integer :: i
    handle = 0
    forgiving = .false.
    if (present(tolerant)) forgiving = tolerant
    keep = .false.
    if (present(persistent)) keep = persistent
    if (size(values) == 0 .or. .not. is_contiguous(values)) then
      if (forgiving) return
      error stop 'an empty or strided array cannot be kept on the device'
    endif
    if (.not. self%active) error stop 'registration outside a storage epoch'
    extents = shape(values, kind=c_size_t)
    bounds = int(lower, c_int64_t)
    identity = transfer(c_loc(values), identity)
    do i = 1, size(self%storage)
      if (self%storage(i)%identity /= identity) cycle
      if (size(self%storage(i)%extents) /= size(extents)) then
        if (forgiving) return
        error stop 'storage rank changed inside an epoch'
      endif
      if (any(self%storage(i)%extents /= extents)) then
        if (forgiving) return
        error stop 'storage shape changed inside an epoch'
      endif
      handle = self%storage(i)%handle
      return
    enddo
    layout%rank = size(extents)
    layout%element_type = FORT_SCOPE_REAL64
    layout%element_bytes = 8
    layout%host = c_loc(values)
    layout%extents = c_loc(extents)
    layout%lower_bounds = c_loc(bounds)
    generation = self%generation
    if (keep) generation = 1
    layout%generation = generation
    call resident_require(fort_scope_register(self%context, identity, generation, layout, &
                                              merge(1_c_int, 0_c_int, initialized), handle))
    item%identity = identity
    item%handle = handle
    item%extents = extents
    item%lower = bounds
    item%persistent = keep
    self%storage = [self%storage, item]
    if (present(origin)) continue
  end function

  function held(self, values) result(handle)
    class(resident_domain), intent(in) :: self
    real(c_double), target, intent(in) :: values(..)
    integer(c_int64_t) :: handle, identity
    integer :: i
    handle = 0
    if (.not. self%active .or. size(values) == 0) return
    identity = transfer(c_loc(values), identity)
    do i = 1, size(self%storage)
      ! the storage whose bytes contain the array's first element
      if (identity < self%storage(i)%identity) cycle
      if (identity >= self%storage(i)%identity + 8_c_int64_t * int(product(self%storage(i)%extents), c_int64_t)) cycle
      handle = self%storage(i)%handle
      return
    enddo
  end function

  ! Hand arrays (by handle; 0 and repeats ignored) to host code that may change them.
  subroutine host_modify(self, handles)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: handles(:)
    type(fort_scope_access), target :: access
    integer :: i
    access%flags = ior(FORT_SCOPE_READ_ALL, FORT_SCOPE_WRITE_ALL)
    do i = 1, size(handles)
      if (handles(i) == 0 .or. any(handles(:i - 1) == handles(i))) cycle
      call resident_require(fort_scope_host_begin(self%context, handles(i), access))
    enddo
  end subroutine

  ! Hand them back, in reverse order, after the host code.
  subroutine host_done(self, handles)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: handles(:)
    integer :: i
    do i = size(handles), 1, -1
      if (handles(i) == 0 .or. any(handles(:i - 1) == handles(i))) cycle
      call resident_require(fort_scope_host_end(self%context, handles(i)))
    enddo
    self%stamp = self%stamp + 1
  end subroutine

  ! Retire an array's device state without bringing its values home: for a
  ! temporary about to be deallocated.
  subroutine release(self, values)
    class(resident_domain), intent(inout) :: self
    real(c_double), target, intent(in) :: values(..)
    integer(c_int64_t) :: handle
    type(held_storage), allocatable :: kept(:)
    handle = self%held(values)
    if (handle == 0) return
    call resident_require(fort_scope_retire_v1(self%context, handle))
    kept = pack(self%storage, self%storage%handle /= handle)
    call move_alloc(kept, self%storage)
  end subroutine

  subroutine observe(self, handles)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: handles(:)
    integer(c_int64_t), allocatable, target :: distinct(:)
    integer :: i
    allocate(distinct(0))
    do i = 1, size(handles)
      if (handles(i) /= 0 .and. .not. any(distinct == handles(i))) distinct = [distinct, handles(i)]
    enddo
    if (size(distinct) == 0) return
    call resident_require(fort_scope_observe_v1(self%context, c_loc(distinct), size(distinct, kind=c_size_t)))
    self%stamp = self%stamp + 1
  end subroutine

  subroutine observe_field(self, first)
    class(resident_domain), intent(inout) :: self
    type(c_ptr), intent(in) :: first
    ! no field of an array of derived type is ever bound here: nothing to bring back
  end subroutine

  subroutine publish(self)
    class(resident_domain), intent(inout) :: self
    type(held_storage), allocatable :: kept(:)
    integer(c_int64_t), allocatable :: handles(:)
    integer :: i
    if (.not. allocated(self%storage)) return
    handles = pack(self%storage%handle, .not. self%storage%persistent)
    call self%observe(handles)
    do i = 1, size(handles)
      call resident_require(fort_scope_unregister(self%context, handles(i)))
    enddo
    kept = pack(self%storage, self%storage%persistent)
    call move_alloc(kept, self%storage)
    self%stamp = self%stamp + 1
  end subroutine

  subroutine end_epoch(self)
    class(resident_domain), intent(inout) :: self
    if (.not. self%active) return
    call self%publish()
    self%active = .false.
  end subroutine

  subroutine close(self)
    class(resident_domain), intent(inout) :: self
    if (self%active) call self%end_epoch()
    if (self%context /= 0) then
      call resident_require(fort_scope_close(self%context))
      call resident_require(fort_scope_domain_close_v1(self%domain))
    endif
    self%context = 0
    self%domain = 0
    if (allocated(self%storage)) deallocate(self%storage)
  end subroutine
end module fort_resident_domain
