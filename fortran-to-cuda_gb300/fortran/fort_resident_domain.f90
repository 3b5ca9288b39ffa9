! The residency domain a resident build's directives and call blocks use.
!
! The type's public methods, their names and their dummy arguments are those of
! the reference's module fort_resident_domain (compiler/runtime/resident_domain.f90),
! so that spliced code and application code written against it compile
! unchanged. What each method does:
!
!  * begin_epoch creates the domain and its context on first use (the caller's
!    budget or the runtime's default) and advances the generation; unless the
!    caller keeps its OpenMP team (keep_team), the epoch narrows the team to
!    FORT_RESIDENT_HOST_THREADS when that is set and end_epoch restores it.
!    A build prepared with --fast-fp (preprocessor symbol F2C_FAST_FP) opens
!    its context under the fast-fp numerical contract.
!  * register_storage registers host storage by address, extents, lower bounds
!    and element type, returning the handle already held for that storage
!    within the epoch; bind_real32 / bind_real64 / bind_integer32 (generic
!    bind, bind_real) do so for an array. A tolerant binding answers 0 where
!    the array cannot be kept (empty, strided, or storage that clashes with
!    what is registered), and the statements there stay on the host.
!  * bind_field keeps one numeric field of a rank-one array of derived type as
!    a contiguous copy that the runtime manages like an array; observe and
!    observe_field write a copy the device changed back into the structures;
!    publish drops the copies.
!  * held answers the handle of the storage an array lies in (0 when none);
!    host_begin / host_end bracket host access to one array, host_modify /
!    host_done to several (each named storage once).
!  * release_real32 / release_real64 (generic release_real, release) retire a
!    temporary's device state without bringing its values home.
!  * work_real32_3 / work_real64_3 lend a procedure a temporary array in place
!    of its ALLOCATE (storage kept per source site and shape while the epoch
!    keeps values on the device, an ordinary allocation otherwise), and
!    work_done_* take it back in place of the DEALLOCATE; acquire_work_* and
!    release_work_* are the lending itself.
!  * publish observes and unregisters every non-persistent array; end_epoch
!    publishes and ends the epoch; close releases the context and the domain.
!
! resident_require stops the program on a nonzero status: work that failed
! after it started is never replayed.
module fort_resident_domain
  use, intrinsic :: iso_c_binding
  use, intrinsic :: iso_fortran_env, only: error_unit
  use fort_scoped_memory
  !$ use omp_lib, only: omp_get_max_threads, omp_set_num_threads
  implicit none
  private
  public :: resident_domain, resident_require

  type :: held_storage
    integer(c_int64_t) :: identity = 0, handle = 0
    integer(c_int) :: element_type = 0
    integer(c_size_t) :: element_bytes = 0
    integer(c_size_t), allocatable :: extents(:)
    character(:), allocatable :: origin
    logical :: persistent = .false.
  end type

  ! A temporary lent to a source site: the domain owns the storage until close.
  type :: lent_real32_3
    integer(c_int64_t) :: site = 0, handle = 0
    real(c_float), pointer, contiguous :: values(:,:,:) => null()
    logical :: borrowed = .false.
  end type

  type :: lent_real64_3
    integer(c_int64_t) :: site = 0, handle = 0
    real(c_double), pointer, contiguous :: values(:,:,:) => null()
    logical :: borrowed = .false.
  end type

  ! A contiguous copy of one field of the elements of a rank-one array of derived type.
  type :: field_copy
    integer(c_intptr_t) :: first = 0
    integer(c_size_t) :: stride = 0, count = 0, bytes = 0
    integer(c_int) :: element_type = 0
    integer(c_int64_t) :: handle = 0
    logical :: written = .false.
    integer(c_int32_t), pointer :: integers(:) => null()
    real(c_float), pointer :: singles(:) => null()
    real(c_double), pointer :: doubles(:) => null()
  end type

  type :: resident_domain
    integer(c_int64_t) :: domain = 0, context = 0, generation = 0
    ! Advances whenever host code may have changed bound values (publications, host accesses).
    integer(c_int64_t) :: stamp = 0
    logical :: active = .false.
    integer, private :: outer_threads = 0
    type(held_storage), allocatable, private :: storage(:)
    character(len=96), allocatable, private :: declined_origins(:)
    type(field_copy), allocatable, private :: fields(:)
    ! Copy blocks that landed on memory still registered for a freed array, kept until the next publication.
    type(field_copy), allocatable, private :: set_aside(:)
    type(lent_real32_3), allocatable, private :: lent32(:)
    type(lent_real64_3), allocatable, private :: lent64(:)
  contains
    procedure :: begin_epoch
    procedure :: unclaimed
    procedure :: register_storage
    procedure :: bind_real32
    procedure :: bind_real64
    generic :: bind_real => bind_real32, bind_real64
    procedure :: bind_integer32
    generic :: bind => bind_real32, bind_real64, bind_integer32
    procedure :: bind_field
    procedure :: observe_field
    procedure :: held
    procedure :: observe
    procedure :: host_begin
    procedure :: host_end
    procedure :: host_modify
    procedure :: host_done
    procedure :: release_real32
    procedure :: release_real64
    generic :: release_real => release_real32, release_real64
    generic :: release => release_real32, release_real64
    procedure :: acquire_work_real32_3
    procedure :: acquire_work_real64_3
    generic :: acquire_work_real_3 => acquire_work_real32_3, acquire_work_real64_3
    procedure :: release_work_real32_3
    procedure :: release_work_real64_3
    generic :: release_work_real_3 => release_work_real32_3, release_work_real64_3
    procedure :: work_real32_3
    procedure :: work_real64_3
    generic :: work => work_real32_3, work_real64_3
    procedure :: work_done_real32_3
    procedure :: work_done_real64_3
    generic :: work_done => work_done_real32_3, work_done_real64_3
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

  subroutine begin_epoch(self, device, budget, keep_team)
    class(resident_domain), intent(inout) :: self
    integer(c_int), intent(in) :: device
    integer(c_size_t), optional, intent(in) :: budget
    logical, optional, intent(in) :: keep_team
    integer(c_size_t) :: bytes
    logical :: keep
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
#ifdef F2C_FAST_FP
      call resident_require(fort_scope_numerics_set_v1(self%context, FORT_SCOPE_NUMERICS_FAST))
#endif
      allocate(self%storage(0))
    endif
    if (self%generation == huge(self%generation)) error stop 'storage generation overflow'
    self%generation = self%generation + 1
    self%active = .true.
    keep = .false.
    if (present(keep_team)) keep = keep_team
    if (.not. keep) call narrow_team(self)
  end subroutine

  ! Between kernels the host runs serial code; every parallel region it still
  ! enters wakes the whole OpenMP team. An epoch therefore narrows the team to
  ! FORT_RESIDENT_HOST_THREADS, when that is set below the current count, and
  ! end_epoch gives the application its own count back.
  subroutine narrow_team(self)
    class(resident_domain), intent(inout) :: self
    character(len=32) :: text
    integer :: wanted, status
    call get_environment_variable('FORT_RESIDENT_HOST_THREADS', text, status=status)
    if (status /= 0) return
    read(text, *, iostat=status) wanted
    if (status /= 0 .or. wanted < 1) error stop 'FORT_RESIDENT_HOST_THREADS must be a positive integer'
    !$ if (wanted < omp_get_max_threads()) then
    !$   self%outer_threads = omp_get_max_threads()
    !$   call omp_set_num_threads(wanted)
    !$ endif
  end subroutine

  function unclaimed(self) result(bytes)
    class(resident_domain), intent(in) :: self
    integer(c_size_t) :: bytes, budget
    if (self%domain == 0) error stop 'budget of a domain that has no epoch yet'
    call resident_require(fort_scope_domain_budget_get_v1(self%domain, budget, bytes))
  end function

  ! Host storage by address. With `collision` present, `host` is a block the
  ! caller has just allocated for itself, so storage registered at it belongs to
  ! an array that no longer exists: no handle, and collision is set. With
  ! `declined` present, storage that cannot be kept as asked (empty, another
  ! shape or type, or memory shared with registered storage) is no error: no
  ! handle, declined is set, and the first refusal at each origin is reported.
  function register_storage(self, host, extents, lower, element_type, element_bytes, initialized, persistent, origin, &
                            collision, declined) result(handle)
    class(resident_domain), intent(inout) :: self
    type(c_ptr), intent(in) :: host
    integer(c_size_t), target, intent(in) :: extents(:)
    integer(c_int64_t), target, intent(in) :: lower(:)
    integer(c_int), intent(in) :: element_type
    integer(c_size_t), intent(in) :: element_bytes
    logical, intent(in) :: initialized, persistent
    character(*), optional, intent(in) :: origin
    logical, optional, intent(out) :: collision, declined
    integer(c_int64_t) :: handle, identity, generation
    type(fort_scope_layout) :: layout
    type(held_storage) :: item
    integer(c_int) :: status
    character(:), allocatable :: place
    integer :: i
    handle = 0
    if (present(collision)) collision = .false.
    if (present(declined)) declined = .false.
    place = 'unknown'
    if (present(origin)) place = origin
    if (.not. self%active) error stop 'registration outside a storage epoch'
    if (size(extents) /= size(lower)) error stop 'invalid resident allocation'
    if (any(extents == 0) .or. .not. c_associated(host)) then
      if (.not. present(declined)) error stop 'invalid or empty resident allocation'
      declined = .true.
      return
    endif
    identity = transfer(host, identity)
    do i = 1, size(self%storage)
      if (self%storage(i)%identity /= identity) cycle
      if (present(collision)) then
        collision = .true.
        return
      endif
      if (self%storage(i)%element_type /= element_type .or. self%storage(i)%element_bytes /= element_bytes .or. &
          (persistent .and. .not. self%storage(i)%persistent)) then
        if (refused(self, place, identity, product(extents) * element_bytes, declined)) return
        error stop 'storage contract changed inside an epoch'
      endif
      if (size(self%storage(i)%extents) /= size(extents)) then
        if (refused(self, place, identity, product(extents) * element_bytes, declined)) return
        error stop 'storage rank changed inside an epoch'
      endif
      if (any(self%storage(i)%extents /= extents)) then
        if (refused(self, place, identity, product(extents) * element_bytes, declined)) return
        error stop 'storage shape changed inside an epoch'
      endif
      if (self%storage(i)%origin == 'unknown') self%storage(i)%origin = place
      handle = self%storage(i)%handle
      return
    enddo
    layout%rank = size(extents)
    layout%element_type = element_type
    layout%element_bytes = element_bytes
    layout%host = host
    layout%extents = c_loc(extents)
    layout%lower_bounds = c_loc(lower)
    generation = self%generation
    if (persistent) generation = 1
    layout%generation = generation
    status = fort_scope_register(self%context, identity, generation, layout, merge(1_c_int, 0_c_int, initialized), &
                                 handle)
    if (status == FORT_SCOPE_ALIAS) then
      handle = 0
      if (present(collision)) then
        collision = .true.
        return
      endif
      if (refused(self, place, identity, product(extents) * element_bytes, declined)) return
      call report_overlap(self, identity, product(extents) * element_bytes, place)
    endif
    call resident_require(status)
    item%identity = identity
    item%handle = handle
    item%element_type = element_type
    item%element_bytes = element_bytes
    item%extents = extents
    item%persistent = persistent
    item%origin = place
    self%storage = [self%storage, item]
  end function

  ! Whether a refusal is taken as an answer (`declined` present); the first one at a place is reported.
  logical function refused(self, place, address, bytes, declined)
    class(resident_domain), intent(inout) :: self
    character(*), intent(in) :: place
    integer(c_int64_t), intent(in) :: address
    integer(c_size_t), intent(in) :: bytes
    logical, optional, intent(out) :: declined
    character(len=96) :: key
    refused = present(declined)
    if (.not. refused) return
    declined = .true.
    key = place
    if (.not. allocated(self%declined_origins)) allocate(self%declined_origins(0))
    if (any(self%declined_origins == key)) return
    self%declined_origins = [self%declined_origins, key]
    write(error_unit, '(a,a,a)') 'Resident array cannot be kept on the device as it is bound at ', trim(place), &
      '; the statements there run on the host.'
    call report_overlap(self, address, bytes, place)
  end function

  ! Name the registered storage that overlaps `bytes` at `address`.
  subroutine report_overlap(self, address, bytes, place)
    class(resident_domain), intent(in) :: self
    integer(c_int64_t), intent(in) :: address
    integer(c_size_t), intent(in) :: bytes
    character(*), intent(in) :: place
    integer(c_int64_t) :: first, size_bytes
    integer :: i, found
    write(error_unit, '(a,a,a,i0,a,i0,a,i0,a,i0)') 'Resident storage overlap: origin=', place, ' address=', address, &
      ' bytes=', bytes, ' domain=', self%domain, ' epoch=', self%generation
    found = 0
    do i = 1, size(self%storage)
      first = self%storage(i)%identity
      size_bytes = int(product(self%storage(i)%extents) * self%storage(i)%element_bytes, c_int64_t)
      if (address + int(bytes, c_int64_t) <= first .or. first + size_bytes <= address) cycle
      found = found + 1
      write(error_unit, '(a,a,a,i0,a,i0,a,l1)') '  registered: origin=', self%storage(i)%origin, ' address=', first, &
        ' bytes=', size_bytes, ' persistent=', self%storage(i)%persistent
    enddo
    if (found == 0) write(error_unit, '(a)') '  registered: by storage this domain has no record of'
  end subroutine

  ! An array by the address of its first element, its extents and lower bounds; contiguity is asked here.
  function bind_storage(self, address, extents, empty, contiguous, lower, element_type, element_bytes, initialized, &
                        persistent, origin, tolerant) result(handle)
    class(resident_domain), intent(inout) :: self
    type(c_ptr), intent(in) :: address
    integer(c_size_t), intent(in) :: extents(:)
    logical, intent(in) :: empty, contiguous
    integer, intent(in) :: lower(:)
    integer(c_int), intent(in) :: element_type
    integer(c_size_t), intent(in) :: element_bytes
    logical, intent(in) :: initialized
    logical, optional, intent(in) :: persistent, tolerant
    character(*), optional, intent(in) :: origin
    integer(c_int64_t) :: handle
    logical :: keep, forgiving, declined
    handle = 0
    forgiving = .false.
    if (present(tolerant)) forgiving = tolerant
    keep = .false.
    if (present(persistent)) keep = persistent
    if (forgiving .and. (empty .or. .not. contiguous)) return
    if (.not. contiguous) error stop 'a strided array section cannot be kept on the device'
    if (forgiving) then
      handle = self%register_storage(address, extents, int(lower, c_int64_t), element_type, element_bytes, &
                                     initialized, keep, origin, declined=declined)
    else
      handle = self%register_storage(address, extents, int(lower, c_int64_t), element_type, element_bytes, &
                                     initialized, keep, origin)
    endif
  end function

  function bind_real32(self, values, lower, initialized, persistent, origin, tolerant) result(handle)
    class(resident_domain), intent(inout) :: self
    real(c_float), target, intent(in) :: values(..)
    integer, intent(in) :: lower(:)
    logical, intent(in) :: initialized
    logical, optional, intent(in) :: persistent
    character(*), optional, intent(in) :: origin
    logical, optional, intent(in) :: tolerant
    integer(c_int64_t) :: handle
    type(c_ptr) :: address
    address = c_null_ptr  ! C_LOC takes no zero-sized or strided array
    if (size(values) > 0 .and. is_contiguous(values)) address = c_loc(values)
    handle = bind_storage(self, address, shape(values, kind=c_size_t), size(values) == 0, &
                          is_contiguous(values), lower, FORT_SCOPE_REAL32, 4_c_size_t, initialized, persistent, &
                          origin, tolerant)
  end function

  function bind_real64(self, values, lower, initialized, persistent, origin, tolerant) result(handle)
    class(resident_domain), intent(inout) :: self
    real(c_double), target, intent(in) :: values(..)
    integer, intent(in) :: lower(:)
    logical, intent(in) :: initialized
    logical, optional, intent(in) :: persistent
    character(*), optional, intent(in) :: origin
    logical, optional, intent(in) :: tolerant
    integer(c_int64_t) :: handle
    type(c_ptr) :: address
    address = c_null_ptr  ! C_LOC takes no zero-sized or strided array
    if (size(values) > 0 .and. is_contiguous(values)) address = c_loc(values)
    handle = bind_storage(self, address, shape(values, kind=c_size_t), size(values) == 0, &
                          is_contiguous(values), lower, FORT_SCOPE_REAL64, 8_c_size_t, initialized, persistent, &
                          origin, tolerant)
  end function

  function bind_integer32(self, values, lower, initialized, persistent, origin, tolerant) result(handle)
    class(resident_domain), intent(inout) :: self
    integer(c_int), target, intent(in) :: values(..)
    integer, intent(in) :: lower(:)
    logical, intent(in) :: initialized
    logical, optional, intent(in) :: persistent
    character(*), optional, intent(in) :: origin
    logical, optional, intent(in) :: tolerant
    integer(c_int64_t) :: handle
    type(c_ptr) :: address
    address = c_null_ptr  ! C_LOC takes no zero-sized or strided array
    if (size(values) > 0 .and. is_contiguous(values)) address = c_loc(values)
    handle = bind_storage(self, address, shape(values, kind=c_size_t), size(values) == 0, &
                          is_contiguous(values), lower, FORT_SCOPE_INTEGER32, 4_c_size_t, initialized, persistent, &
                          origin, tolerant)
  end function

  ! The handle of the registered storage holding the first of these values (0 when none does).
  function held(self, values) result(handle)
    class(resident_domain), intent(in) :: self
    type(*), target, intent(in) :: values(..)
    integer(c_int64_t) :: handle, address, first
    integer :: i
    handle = 0
    if (.not. self%active) return
    if (size(values) == 0 .or. .not. is_contiguous(values)) return
    address = transfer(c_loc(values), address)
    do i = 1, size(self%storage)
      first = self%storage(i)%identity
      if (address < first) cycle
      if (address >= first + int(product(self%storage(i)%extents) * self%storage(i)%element_bytes, c_int64_t)) cycle
      handle = self%storage(i)%handle
      return
    enddo
  end function

  ! Each nonzero handle once.
  pure function distinct(handles) result(found)
    integer(c_int64_t), intent(in) :: handles(:)
    integer(c_int64_t), allocatable :: found(:)
    integer :: i
    allocate(found(0))
    do i = 1, size(handles)
      if (handles(i) /= 0 .and. .not. any(found == handles(i))) found = [found, handles(i)]
    enddo
  end function

  subroutine observe(self, handles)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: handles(:)
    integer(c_int64_t), allocatable, target :: bound(:)
    integer :: i
    bound = distinct(handles)
    if (size(bound) == 0) return
    call resident_require(fort_scope_observe_v1(self%context, c_loc(bound), size(bound, kind=c_size_t)))
    self%stamp = self%stamp + 1
    if (.not. allocated(self%fields)) return
    do i = 1, size(self%fields)
      if (self%fields(i)%written .and. any(bound == self%fields(i)%handle)) call move_field(self%fields(i), .false.)
    enddo
  end subroutine

  ! One field of an array of derived type, by the address of the field in its first element.
  subroutine observe_field(self, first)
    class(resident_domain), intent(inout) :: self
    type(c_ptr), intent(in) :: first
    integer :: i
    if (.not. allocated(self%fields)) return
    do i = 1, size(self%fields)
      if (self%fields(i)%first == transfer(first, self%fields(i)%first)) call self%observe([self%fields(i)%handle])
    enddo
  end subroutine

  function copy_address(copy) result(address)
    type(field_copy), intent(in) :: copy
    type(c_ptr) :: address
    select case (copy%element_type)
    case (FORT_SCOPE_INTEGER32)
      address = c_loc(copy%integers)
    case (FORT_SCOPE_REAL32)
      address = c_loc(copy%singles)
    case default
      address = c_loc(copy%doubles)
    end select
  end function

  ! Gather the field from the structures into the copy, or scatter the copy back.
  subroutine move_field(copy, gather)
    type(field_copy), intent(in) :: copy
    logical, intent(in) :: gather
    integer(c_int8_t), pointer :: structures(:), values(:)
    integer(c_size_t) :: n, at, from
    call c_f_pointer(transfer(copy%first, c_null_ptr), structures, [(copy%count - 1) * copy%stride + copy%bytes])
    call c_f_pointer(copy_address(copy), values, [copy%count * copy%bytes])
    do n = 0, copy%count - 1
      at = n * copy%bytes
      from = n * copy%stride
      if (gather) then
        values(at + 1:at + copy%bytes) = structures(from + 1:from + copy%bytes)
      else
        structures(from + 1:from + copy%bytes) = values(at + 1:at + copy%bytes)
      endif
    enddo
  end subroutine

  subroutine free_copies(copies)
    type(field_copy), allocatable, intent(inout) :: copies(:)
    integer :: i
    do i = 1, size(copies)
      if (associated(copies(i)%integers)) deallocate(copies(i)%integers)
      if (associated(copies(i)%singles)) deallocate(copies(i)%singles)
      if (associated(copies(i)%doubles)) deallocate(copies(i)%doubles)
    enddo
    deallocate(copies)
  end subroutine

  ! One field of every element of a rank-one array of derived type: `first` is
  ! the field's address in the first element, `stride` an element's size in
  ! bytes. The values are copied from the structures when the field is first
  ! bound and stay bound until the next publication.
  function bind_field(self, first, stride, count, element_type, writing, origin) result(handle)
    class(resident_domain), intent(inout) :: self
    type(c_ptr), intent(in) :: first
    integer(c_size_t), intent(in) :: stride, count
    integer(c_int), intent(in) :: element_type
    logical, intent(in) :: writing
    character(*), optional, intent(in) :: origin
    integer(c_int64_t) :: handle
    ! the memory one binding may set aside while it looks for a block no registration covers
    integer(c_size_t), parameter :: set_aside_limit = 1073741824_c_size_t
    type(field_copy) :: item
    integer(c_size_t) :: aside
    logical :: collision
    integer :: i
    if (.not. self%active) error stop 'field binding outside a storage epoch'
    if (count == 0 .or. .not. c_associated(first)) error stop 'invalid or empty resident field'
    if (.not. allocated(self%fields)) allocate(self%fields(0))
    item%first = transfer(first, item%first)
    do i = 1, size(self%fields)
      if (self%fields(i)%first /= item%first) cycle
      if (self%fields(i)%stride /= stride .or. self%fields(i)%count /= count .or. &
          self%fields(i)%element_type /= element_type) error stop 'field layout changed inside an epoch'
      self%fields(i)%written = self%fields(i)%written .or. writing
      handle = self%fields(i)%handle
      return
    enddo
    item%stride = stride
    item%count = count
    item%element_type = element_type
    item%written = writing
    select case (element_type)
    case (FORT_SCOPE_INTEGER32, FORT_SCOPE_REAL32)
      item%bytes = 4
    case (FORT_SCOPE_REAL64)
      item%bytes = 8
    case default
      error stop 'unsupported resident field type'
    end select
    if (stride < item%bytes) error stop 'invalid resident field stride'
    aside = 0
    do
      select case (element_type)
      case (FORT_SCOPE_INTEGER32)
        allocate(item%integers(count))
      case (FORT_SCOPE_REAL32)
        allocate(item%singles(count))
      case default
        allocate(item%doubles(count))
      end select
      call move_field(item, .true.)
      item%handle = self%register_storage(copy_address(item), [count], [1_c_int64_t], element_type, item%bytes, &
                                          .true., .false., origin, collision)
      if (.not. collision) exit
      ! The allocator handed out memory still registered for an array its owner freed: keep this block out of
      ! circulation until the next publication and take another.
      if (.not. allocated(self%set_aside)) allocate(self%set_aside(0))
      self%set_aside = [self%set_aside, item]
      nullify(item%integers, item%singles, item%doubles)
      aside = aside + count * item%bytes
      if (aside > set_aside_limit) error stop 'no host memory free of stale registrations for a resident field'
    enddo
    self%fields = [self%fields, item]
    handle = item%handle
  end function

  subroutine host_begin(self, handle, access)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: handle
    type(fort_scope_access), intent(in) :: access
    self%stamp = self%stamp + 1
    call resident_require(fort_scope_host_begin(self%context, handle, access))
  end subroutine

  subroutine host_end(self, handle)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: handle
    call resident_require(fort_scope_host_end(self%context, handle))
  end subroutine

  ! Host statements are about to read and change these arrays anywhere.
  subroutine host_modify(self, handles)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: handles(:)
    integer(c_int64_t), allocatable :: bound(:)
    type(fort_scope_access) :: access
    integer :: i
    access%flags = ior(FORT_SCOPE_READ_ALL, FORT_SCOPE_WRITE_ALL)
    bound = distinct(handles)
    do i = 1, size(bound)
      call self%host_begin(bound(i), access)
    enddo
  end subroutine

  ! ... and are done: hand them back, in reverse order.
  subroutine host_done(self, handles)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: handles(:)
    integer(c_int64_t), allocatable :: bound(:)
    integer :: i
    bound = distinct(handles)
    do i = size(bound), 1, -1
      call self%host_end(bound(i))
    enddo
    self%stamp = self%stamp + 1
  end subroutine

  ! Retire the storage at `address` (a temporary about to be deallocated): its values are dead, nothing moves.
  subroutine retire_at(self, address)
    class(resident_domain), intent(inout) :: self
    type(c_ptr), intent(in) :: address
    integer(c_int64_t) :: identity
    logical, allocatable :: keep(:)
    integer :: i
    if (.not. self%active) return
    identity = transfer(address, identity)
    do i = 1, size(self%storage)
      if (self%storage(i)%identity /= identity) cycle
      if (self%storage(i)%persistent) error stop 'persistent storage retired through a borrowed view'
      call resident_require(fort_scope_retire_v1(self%context, self%storage(i)%handle))
      allocate(keep(size(self%storage)))
      keep = .true.
      keep(i) = .false.
      self%storage = pack(self%storage, keep)
      return
    enddo
  end subroutine

  subroutine release_real32(self, values)
    class(resident_domain), intent(inout) :: self
    real(c_float), target, intent(in) :: values(..)
    if (size(values) == 0 .or. .not. is_contiguous(values)) return
    call retire_at(self, c_loc(values))
  end subroutine

  subroutine release_real64(self, values)
    class(resident_domain), intent(inout) :: self
    real(c_double), target, intent(in) :: values(..)
    if (size(values) == 0 .or. .not. is_contiguous(values)) return
    call retire_at(self, c_loc(values))
  end subroutine

  ! Lend the storage of `site` for this shape: a slot no call still holds is
  ! reused (its values dead, replaced in queue order by the borrower's writes),
  ! else a new persistent slot is made.
  subroutine acquire_work_real32_3(self, site, lower, upper, values)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: site
    integer, intent(in) :: lower(3), upper(3)
    real(c_float), pointer, contiguous, intent(out) :: values(:,:,:)
    type(lent_real32_3) :: slot
    integer :: i
    if (.not. self%active .or. site == 0) error stop 'workspace outside a checked epoch'
    if (any(upper < lower)) error stop 'empty workspace must be skipped by its reached caller'
    if (.not. allocated(self%lent32)) allocate(self%lent32(0))
    do i = 1, size(self%lent32)
      if (self%lent32(i)%site /= site .or. self%lent32(i)%borrowed) cycle
      if (any(lbound(self%lent32(i)%values) /= lower) .or. any(ubound(self%lent32(i)%values) /= upper)) cycle
      call resident_require(fort_scope_recycle_v1(self%context, self%lent32(i)%handle))
      self%lent32(i)%borrowed = .true.
      values => self%lent32(i)%values
      return
    enddo
    slot%site = site
    allocate(slot%values(lower(1):upper(1), lower(2):upper(2), lower(3):upper(3)))
    slot%handle = self%bind_real32(slot%values, lower, .false., persistent=.true.)
    slot%borrowed = .true.
    self%lent32 = [self%lent32, slot]
    values => slot%values
  end subroutine

  subroutine acquire_work_real64_3(self, site, lower, upper, values)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: site
    integer, intent(in) :: lower(3), upper(3)
    real(c_double), pointer, contiguous, intent(out) :: values(:,:,:)
    type(lent_real64_3) :: slot
    integer :: i
    if (.not. self%active .or. site == 0) error stop 'workspace outside a checked epoch'
    if (any(upper < lower)) error stop 'empty workspace must be skipped by its reached caller'
    if (.not. allocated(self%lent64)) allocate(self%lent64(0))
    do i = 1, size(self%lent64)
      if (self%lent64(i)%site /= site .or. self%lent64(i)%borrowed) cycle
      if (any(lbound(self%lent64(i)%values) /= lower) .or. any(ubound(self%lent64(i)%values) /= upper)) cycle
      call resident_require(fort_scope_recycle_v1(self%context, self%lent64(i)%handle))
      self%lent64(i)%borrowed = .true.
      values => self%lent64(i)%values
      return
    enddo
    slot%site = site
    allocate(slot%values(lower(1):upper(1), lower(2):upper(2), lower(3):upper(3)))
    slot%handle = self%bind_real64(slot%values, lower, .false., persistent=.true.)
    slot%borrowed = .true.
    self%lent64 = [self%lent64, slot]
    values => slot%values
  end subroutine

  subroutine release_work_real32_3(self, site, values)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: site
    real(c_float), pointer, contiguous, intent(inout) :: values(:,:,:)
    integer :: i
    if (.not. self%active .or. .not. associated(values) .or. .not. allocated(self%lent32)) &
      error stop 'invalid compiler workspace release'
    do i = 1, size(self%lent32)
      if (self%lent32(i)%site /= site .or. .not. associated(values, self%lent32(i)%values)) cycle
      if (.not. self%lent32(i)%borrowed) error stop 'compiler workspace released twice'
      self%lent32(i)%borrowed = .false.
      nullify(values)
      return
    enddo
    error stop 'foreign compiler workspace release'
  end subroutine

  subroutine release_work_real64_3(self, site, values)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: site
    real(c_double), pointer, contiguous, intent(inout) :: values(:,:,:)
    integer :: i
    if (.not. self%active .or. .not. associated(values) .or. .not. allocated(self%lent64)) &
      error stop 'invalid compiler workspace release'
    do i = 1, size(self%lent64)
      if (self%lent64(i)%site /= site .or. .not. associated(values, self%lent64(i)%values)) cycle
      if (.not. self%lent64(i)%borrowed) error stop 'compiler workspace released twice'
      self%lent64(i)%borrowed = .false.
      nullify(values)
      return
    enddo
    error stop 'foreign compiler workspace release'
  end subroutine

  ! In place of a temporary's ALLOCATE: lent storage while the epoch keeps values on the device, else allocated.
  subroutine work_real32_3(self, site, lower, upper, values)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: site
    integer, intent(in) :: lower(3), upper(3)
    real(c_float), pointer, contiguous, intent(out) :: values(:,:,:)
    if (self%active .and. all(upper >= lower)) then
      call self%acquire_work_real32_3(site, lower, upper, values)
    else
      allocate(values(lower(1):upper(1), lower(2):upper(2), lower(3):upper(3)))
    endif
  end subroutine

  subroutine work_real64_3(self, site, lower, upper, values)
    class(resident_domain), intent(inout) :: self
    integer(c_int64_t), intent(in) :: site
    integer, intent(in) :: lower(3), upper(3)
    real(c_double), pointer, contiguous, intent(out) :: values(:,:,:)
    if (self%active .and. all(upper >= lower)) then
      call self%acquire_work_real64_3(site, lower, upper, values)
    else
      allocate(values(lower(1):upper(1), lower(2):upper(2), lower(3):upper(3)))
    endif
  end subroutine

  ! In place of its DEALLOCATE: lent storage goes back with its values dead, anything else is deallocated.
  subroutine work_done_real32_3(self, values)
    class(resident_domain), intent(inout) :: self
    real(c_float), pointer, contiguous, intent(inout) :: values(:,:,:)
    integer :: i
    if (allocated(self%lent32)) then
      do i = 1, size(self%lent32)
        if (.not. associated(values, self%lent32(i)%values)) cycle
        self%lent32(i)%borrowed = .false.
        nullify(values)
        return
      enddo
    endif
    deallocate(values)
  end subroutine

  subroutine work_done_real64_3(self, values)
    class(resident_domain), intent(inout) :: self
    real(c_double), pointer, contiguous, intent(inout) :: values(:,:,:)
    integer :: i
    if (allocated(self%lent64)) then
      do i = 1, size(self%lent64)
        if (.not. associated(values, self%lent64(i)%values)) cycle
        self%lent64(i)%borrowed = .false.
        nullify(values)
        return
      enddo
    endif
    deallocate(values)
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
    ! the structures hold their fields again
    if (allocated(self%fields)) call free_copies(self%fields)
    if (allocated(self%set_aside)) call free_copies(self%set_aside)
    self%stamp = self%stamp + 1
  end subroutine

  subroutine end_epoch(self)
    class(resident_domain), intent(inout) :: self
    if (allocated(self%lent32)) then
      if (any(self%lent32%borrowed)) error stop 'unmanaged return with borrowed workspace'
    endif
    if (allocated(self%lent64)) then
      if (any(self%lent64%borrowed)) error stop 'unmanaged return with borrowed workspace'
    endif
    call self%publish()
    self%active = .false.
    !$ if (self%outer_threads > 0) call omp_set_num_threads(self%outer_threads)
    self%outer_threads = 0
  end subroutine

  subroutine close(self)
    class(resident_domain), intent(inout) :: self
    integer :: i
    if (self%domain == 0) return
    call self%end_epoch()
    ! lent storage holds dead values: discard them (the domain's close waits for their queued users)
    if (allocated(self%lent32)) then
      do i = 1, size(self%lent32)
        call resident_require(fort_scope_discard_v1(self%context, self%lent32(i)%handle))
      enddo
    endif
    if (allocated(self%lent64)) then
      do i = 1, size(self%lent64)
        call resident_require(fort_scope_discard_v1(self%context, self%lent64(i)%handle))
      enddo
    endif
    call resident_require(fort_scope_close(self%context))
    call resident_require(fort_scope_domain_close_v1(self%domain))
    if (allocated(self%lent32)) then
      do i = 1, size(self%lent32)
        deallocate(self%lent32(i)%values)
      enddo
      deallocate(self%lent32)
    endif
    if (allocated(self%lent64)) then
      do i = 1, size(self%lent64)
        deallocate(self%lent64(i)%values)
      enddo
      deallocate(self%lent64)
    endif
    self%context = 0
    self%domain = 0
    if (allocated(self%storage)) deallocate(self%storage)
  end subroutine
end module fort_resident_domain
