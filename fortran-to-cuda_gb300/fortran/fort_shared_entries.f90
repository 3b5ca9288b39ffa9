! Fortran interfaces of the GB300 numerical entries (generated by compiler/emission).
! One module per entry, the shape of the reference's shared_interface.f90

module fort_shared_ce4761579065
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, arr_handle, val, unx, uny, unz) bind(C, name='cpp_fort_shared_ce4761579065') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: arr_handle
      real(c_double), intent(in) :: val
      integer(c_int), intent(in) :: unx
      integer(c_int), intent(in) :: uny
      integer(c_int), intent(in) :: unz
    end function
  end interface
end module fort_shared_ce4761579065

module fort_shared_79b994dd0404
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, arr_handle, val, unx, uny, unz) bind(C, name='cpp_fort_shared_79b994dd0404') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: arr_handle
      real(c_double), intent(in) :: val
      integer(c_int), intent(in) :: unx
      integer(c_int), intent(in) :: uny
      integer(c_int), intent(in) :: unz
    end function
  end interface
end module fort_shared_79b994dd0404

module fort_shared_c332ebf80d68
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u2_handle, u_handle, v_handle, w_handle, dxmin, dymin, dzmin, unx, &
      uny, unz) bind(C, name='cpp_fort_shared_c332ebf80d68') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dxmin
      real(c_double), intent(in) :: dymin
      real(c_double), intent(in) :: dzmin
      integer(c_int), intent(in) :: unx
      integer(c_int), intent(in) :: uny
      integer(c_int), intent(in) :: unz
    end function
  end interface
end module fort_shared_c332ebf80d68

module fort_shared_ae1df5b16148
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u2_handle, u_handle, v_handle, w_handle, dxmin, dymin, dzmin, unx, &
      uny, unz) bind(C, name='cpp_fort_shared_ae1df5b16148') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dxmin
      real(c_double), intent(in) :: dymin
      real(c_double), intent(in) :: dzmin
      integer(c_int), intent(in) :: unx
      integer(c_int), intent(in) :: uny
      integer(c_int), intent(in) :: unz
    end function
  end interface
end module fort_shared_ae1df5b16148

module fort_shared_42de9862e2fe
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u2_handle, u_handle, v_handle, w_handle, dxmin, dymin, dzmin, unx, &
      uny, unz) bind(C, name='cpp_fort_shared_42de9862e2fe') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dxmin
      real(c_double), intent(in) :: dymin
      real(c_double), intent(in) :: dzmin
      integer(c_int), intent(in) :: unx
      integer(c_int), intent(in) :: uny
      integer(c_int), intent(in) :: unz
    end function
  end interface
end module fort_shared_42de9862e2fe

module fort_shared_dc5f61a1cb0a
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, v2_handle, u_handle, v_handle, w_handle, dxmin, dymin, dzmin, vnx, &
      vny, vnz) bind(C, name='cpp_fort_shared_dc5f61a1cb0a') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: v2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dxmin
      real(c_double), intent(in) :: dymin
      real(c_double), intent(in) :: dzmin
      integer(c_int), intent(in) :: vnx
      integer(c_int), intent(in) :: vny
      integer(c_int), intent(in) :: vnz
    end function
  end interface
end module fort_shared_dc5f61a1cb0a

module fort_shared_4091fbf13dda
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, v2_handle, u_handle, v_handle, w_handle, dxmin, dymin, dzmin, vnx, &
      vny, vnz) bind(C, name='cpp_fort_shared_4091fbf13dda') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: v2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dxmin
      real(c_double), intent(in) :: dymin
      real(c_double), intent(in) :: dzmin
      integer(c_int), intent(in) :: vnx
      integer(c_int), intent(in) :: vny
      integer(c_int), intent(in) :: vnz
    end function
  end interface
end module fort_shared_4091fbf13dda

module fort_shared_a72cc49a3bc2
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, v2_handle, u_handle, v_handle, w_handle, dxmin, dymin, dzmin, vnx, &
      vny, vnz) bind(C, name='cpp_fort_shared_a72cc49a3bc2') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: v2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dxmin
      real(c_double), intent(in) :: dymin
      real(c_double), intent(in) :: dzmin
      integer(c_int), intent(in) :: vnx
      integer(c_int), intent(in) :: vny
      integer(c_int), intent(in) :: vnz
    end function
  end interface
end module fort_shared_a72cc49a3bc2

module fort_shared_1664ef72e5f6
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, w2_handle, u_handle, v_handle, w_handle, dxmin, dymin, dzmin, wnx, &
      wny, wnz) bind(C, name='cpp_fort_shared_1664ef72e5f6') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: w2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dxmin
      real(c_double), intent(in) :: dymin
      real(c_double), intent(in) :: dzmin
      integer(c_int), intent(in) :: wnx
      integer(c_int), intent(in) :: wny
      integer(c_int), intent(in) :: wnz
    end function
  end interface
end module fort_shared_1664ef72e5f6

module fort_shared_93e5f62400e4
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, w2_handle, u_handle, v_handle, w_handle, dxmin, dymin, dzmin, wnx, &
      wny, wnz) bind(C, name='cpp_fort_shared_93e5f62400e4') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: w2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dxmin
      real(c_double), intent(in) :: dymin
      real(c_double), intent(in) :: dzmin
      integer(c_int), intent(in) :: wnx
      integer(c_int), intent(in) :: wny
      integer(c_int), intent(in) :: wnz
    end function
  end interface
end module fort_shared_93e5f62400e4

module fort_shared_a28440d2f301
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, w2_handle, u_handle, v_handle, w_handle, dxmin, dymin, dzmin, wnx, &
      wny, wnz) bind(C, name='cpp_fort_shared_a28440d2f301') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: w2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dxmin
      real(c_double), intent(in) :: dymin
      real(c_double), intent(in) :: dzmin
      integer(c_int), intent(in) :: wnx
      integer(c_int), intent(in) :: wny
      integer(c_int), intent(in) :: wnz
    end function
  end interface
end module fort_shared_a28440d2f301

module fort_shared_0e71295b0ec3
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u2_handle, v2_handle, w2_handle, u_handle, v_handle, w_handle, dx, &
      dy, dz, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_0e71295b0ec3') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u2_handle
      integer(c_int64_t), value :: v2_handle
      integer(c_int64_t), value :: w2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_0e71295b0ec3

module fort_shared_001e6a9fcfd6
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, un_handle, vn_handle, wn_handle, u_handle, v_handle, w_handle, dx, &
      dy, dz, dt, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_001e6a9fcfd6') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: un_handle
      integer(c_int64_t), value :: vn_handle
      integer(c_int64_t), value :: wn_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      real(c_double), intent(in) :: dt
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_001e6a9fcfd6

module fort_shared_4d5ee7974150
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u_handle, v_handle, w_handle, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_4d5ee7974150') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_4d5ee7974150

module fort_shared_a5b15bb8130a
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u2_handle, v2_handle, w2_handle, u_handle, v_handle, w_handle, &
      s1_handle, s1t_handle, dx, dy, dz, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_a5b15bb8130a') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u2_handle
      integer(c_int64_t), value :: v2_handle
      integer(c_int64_t), value :: w2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s1t_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_a5b15bb8130a

module fort_shared_45d68b9decbb
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, un_handle, vn_handle, wn_handle, u_handle, v_handle, w_handle, &
      s1_handle, s1n_handle, dx, dy, dz, dt, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_45d68b9decbb') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: un_handle
      integer(c_int64_t), value :: vn_handle
      integer(c_int64_t), value :: wn_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s1n_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      real(c_double), intent(in) :: dt
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_45d68b9decbb

module fort_shared_f5b3f004c0dc
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u_handle, v_handle, w_handle, s1_handle, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_f5b3f004c0dc') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_f5b3f004c0dc

module fort_shared_cac08e022e8e
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u2_handle, v2_handle, w2_handle, u_handle, v_handle, w_handle, &
      s1_handle, s2_handle, s1t_handle, s2t_handle, dx, dy, dz, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_cac08e022e8e') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u2_handle
      integer(c_int64_t), value :: v2_handle
      integer(c_int64_t), value :: w2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s2_handle
      integer(c_int64_t), value :: s1t_handle
      integer(c_int64_t), value :: s2t_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_cac08e022e8e

module fort_shared_405aeb9f9533
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, un_handle, vn_handle, wn_handle, u_handle, v_handle, w_handle, &
      s1_handle, s2_handle, s1n_handle, s2n_handle, dx, dy, dz, dt, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_405aeb9f9533') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: un_handle
      integer(c_int64_t), value :: vn_handle
      integer(c_int64_t), value :: wn_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s2_handle
      integer(c_int64_t), value :: s1n_handle
      integer(c_int64_t), value :: s2n_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      real(c_double), intent(in) :: dt
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_405aeb9f9533

module fort_shared_9f0fa829d5ff
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u_handle, v_handle, w_handle, s1_handle, s2_handle, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_9f0fa829d5ff') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s2_handle
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_9f0fa829d5ff

module fort_shared_c3ee1d88b7ff
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u2_handle, v2_handle, w2_handle, u_handle, v_handle, w_handle, &
      s1_handle, s2_handle, s3_handle, s1t_handle, s2t_handle, s3t_handle, dx, dy, dz, nx, ny, nz, &
      halo) bind(C, name='cpp_fort_shared_c3ee1d88b7ff') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u2_handle
      integer(c_int64_t), value :: v2_handle
      integer(c_int64_t), value :: w2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s2_handle
      integer(c_int64_t), value :: s3_handle
      integer(c_int64_t), value :: s1t_handle
      integer(c_int64_t), value :: s2t_handle
      integer(c_int64_t), value :: s3t_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_c3ee1d88b7ff

module fort_shared_f6ba06adab12
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, un_handle, vn_handle, wn_handle, u_handle, v_handle, w_handle, &
      s1_handle, s2_handle, s3_handle, s1n_handle, s2n_handle, s3n_handle, dx, dy, dz, dt, nx, ny, &
      nz, halo) bind(C, name='cpp_fort_shared_f6ba06adab12') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: un_handle
      integer(c_int64_t), value :: vn_handle
      integer(c_int64_t), value :: wn_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s2_handle
      integer(c_int64_t), value :: s3_handle
      integer(c_int64_t), value :: s1n_handle
      integer(c_int64_t), value :: s2n_handle
      integer(c_int64_t), value :: s3n_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      real(c_double), intent(in) :: dt
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_f6ba06adab12

module fort_shared_4effb4648a3e
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u_handle, v_handle, w_handle, s1_handle, s2_handle, s3_handle, nx, &
      ny, nz, halo) bind(C, name='cpp_fort_shared_4effb4648a3e') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s2_handle
      integer(c_int64_t), value :: s3_handle
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_4effb4648a3e

module fort_shared_6f06b55ba3fe
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u2_handle, v2_handle, w2_handle, u_handle, v_handle, w_handle, &
      s1_handle, s2_handle, s3_handle, s4_handle, s1t_handle, s2t_handle, s3t_handle, s4t_handle, &
      dx, dy, dz, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_6f06b55ba3fe') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u2_handle
      integer(c_int64_t), value :: v2_handle
      integer(c_int64_t), value :: w2_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s2_handle
      integer(c_int64_t), value :: s3_handle
      integer(c_int64_t), value :: s4_handle
      integer(c_int64_t), value :: s1t_handle
      integer(c_int64_t), value :: s2t_handle
      integer(c_int64_t), value :: s3t_handle
      integer(c_int64_t), value :: s4t_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_6f06b55ba3fe

module fort_shared_cbf2341c8e18
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, un_handle, vn_handle, wn_handle, u_handle, v_handle, w_handle, &
      s1_handle, s2_handle, s3_handle, s4_handle, s1n_handle, s2n_handle, s3n_handle, s4n_handle, &
      dx, dy, dz, dt, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_cbf2341c8e18') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: un_handle
      integer(c_int64_t), value :: vn_handle
      integer(c_int64_t), value :: wn_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s2_handle
      integer(c_int64_t), value :: s3_handle
      integer(c_int64_t), value :: s4_handle
      integer(c_int64_t), value :: s1n_handle
      integer(c_int64_t), value :: s2n_handle
      integer(c_int64_t), value :: s3n_handle
      integer(c_int64_t), value :: s4n_handle
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz
      real(c_double), intent(in) :: dt
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_cbf2341c8e18

module fort_shared_073d04efb82a
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, u_handle, v_handle, w_handle, s1_handle, s2_handle, s3_handle, &
      s4_handle, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_073d04efb82a') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: u_handle
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: w_handle
      integer(c_int64_t), value :: s1_handle
      integer(c_int64_t), value :: s2_handle
      integer(c_int64_t), value :: s3_handle
      integer(c_int64_t), value :: s4_handle
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_073d04efb82a

module fort_shared_e331fbb8bf9a
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, b_handle, a_handle, dt, nu, dx, nx, ny, nz, halo) bind(C, name='cpp_fort_shared_e331fbb8bf9a') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: b_handle
      integer(c_int64_t), value :: a_handle
      real(c_double), intent(in) :: dt
      real(c_double), intent(in) :: nu
      real(c_double), intent(in) :: dx
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_e331fbb8bf9a

module fort_shared_03470f69376f
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, v_handle, u_handle, nx, ny, halo) bind(C, name='cpp_fort_shared_03470f69376f') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: v_handle
      integer(c_int64_t), value :: u_handle
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_03470f69376f

module fort_shared_82041a3f2b68
  use iso_c_binding
  implicit none
  private
  public :: run
  interface
    function run( &
      fort_context, fort_mode, ez_handle, hx_handle, hy_handle, ch, ce, nx, ny, halo) bind(C, name='cpp_fort_shared_82041a3f2b68') result(fort_status)
      import :: c_int, c_int64_t, c_double
      integer(c_int) :: fort_status
      integer(c_int64_t), value :: fort_context
      integer(c_int), value :: fort_mode
      integer(c_int64_t), value :: ez_handle
      integer(c_int64_t), value :: hx_handle
      integer(c_int64_t), value :: hy_handle
      real(c_double), intent(in) :: ch
      real(c_double), intent(in) :: ce
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: halo
    end function
  end interface
end module fort_shared_82041a3f2b68
