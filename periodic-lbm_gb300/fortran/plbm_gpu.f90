!> plbm_gpu -- Fortran drop-in for the periodic-lbm hot path on a GB300.
!>
!> Procedures with the reference's interfaces that run the stream/collide
!> hot path on the GPU through libplbmgpu.so (C ABI: include/plbm_gpu.h):
!>
!>   lbm_stream_gpu(grid)       streaming_interface, src/periodic_lbm.f90:32-43
!>   stream_fvm_bardow_gpu(grid), stream_fdm_bardow_gpu(grid),
!>   stream_fdm_sofonea_gpu(grid)  streaming_interface, src/fvm_bardow.F90:393,511,688
!>   collide_bgk_gpu(grid)      collision_interface, src/collision_bgk.F90:17
!>   collide_trt_gpu(grid)      collision_interface, src/collision_trt.F90:41
!>   collide_rr_gpu(grid)       collision_interface, src/collision_regularized.F90:21
!>   collide_bgk_improved_gpu(grid)  src/collision_bgk_improved.f90:16
!>   perform_lbm_step_gpu(grid) src/periodic_lbm.f90:15-29, one fused kernel
!>   perform_triple_step_gpu(grid)  src/fvm_bardow.F90:322-340, one fused kernel
!>   update_macros_gpu(grid)    src/fvm_bardow.F90:343-390
!>   output_npy_gpu(grid[,step])  src/fvm_bardow.F90:930-961, moments of the
!>                              device state written as .npy
!>
!> The lattice lives on the device between calls; grid%f on the host is only
!> read by plbm_gpu_attach / plbm_gpu_upload and written by plbm_gpu_download.
!> A side table keyed by the address of grid%f maps each lattice_grid to its
!> device handle.  grid%iold / grid%inew stay the Fortran's: every call passes
!> them to the handle, so perform_lbm_step's swap keeps working unchanged.
!>
!> Errors: a non-zero status from the library stops the program with the
!> library's message (the reference's error behaviour is `error stop`).
!>
!> This module is compiled together with the reference's src/ (it uses
!> fvm_bardow's lattice_grid).  No Fortran compiler was available where this
!> library was built, so this file has not been compiled; the C ABI it binds
!> is tested from C/Python.
module plbm_gpu

   use, intrinsic :: iso_c_binding, only: c_int, c_double, c_ptr, c_null_ptr, c_loc, &
      c_associated, c_char, c_f_pointer, c_intptr_t, c_null_char
   use precision, only: wp
   use fvm_bardow, only: lattice_grid

   implicit none
   private

   public :: plbm_gpu_attach, plbm_gpu_detach, plbm_gpu_upload, plbm_gpu_download
   public :: lbm_stream_gpu, perform_lbm_step_gpu, update_macros_gpu
   public :: perform_triple_step_gpu, output_npy_gpu
   public :: stream_fvm_bardow_gpu, stream_fdm_bardow_gpu, stream_fdm_sofonea_gpu
   public :: collide_bgk_gpu, collide_trt_gpu, collide_rr_gpu, collide_bgk_improved_gpu
   public :: PLBM_MATH_FMA, PLBM_MATH_STRICT, PLBM_MATH_HYBRID

   integer(c_int), parameter :: PLBM_BGK = 0, PLBM_TRT = 1, PLBM_RR = 2, PLBM_BGKI = 3
   integer(c_int), parameter :: PLBM_F64 = 0
   integer(c_int), parameter :: PLBM_MATH_FMA = 0, PLBM_MATH_STRICT = 1, PLBM_MATH_HYBRID = 2

   interface
      integer(c_int) function plbm_grid_create(nx, ny, nf, storage, out) bind(c, name="plbm_grid_create")
         import :: c_int, c_ptr
         integer(c_int), value :: nx, ny, nf, storage
         type(c_ptr), intent(out) :: out
      end function
      integer(c_int) function plbm_grid_destroy(g) bind(c, name="plbm_grid_destroy")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
      end function
      integer(c_int) function plbm_grid_set_indices(g, iold, inew) bind(c, name="plbm_grid_set_indices")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
         integer(c_int), value :: iold, inew
      end function
      integer(c_int) function plbm_set_relaxation(g, omega, magic) bind(c, name="plbm_set_relaxation")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: g
         real(c_double), value :: omega, magic
      end function
      integer(c_int) function plbm_set_collision(g, kind) bind(c, name="plbm_set_collision")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
         integer(c_int), value :: kind
      end function
      integer(c_int) function plbm_set_math(g, math) bind(c, name="plbm_set_math")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
         integer(c_int), value :: math
      end function
      integer(c_int) function plbm_upload(g, f, ibuf) bind(c, name="plbm_upload")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: g
         real(c_double), intent(in) :: f(*)
         integer(c_int), value :: ibuf
      end function
      integer(c_int) function plbm_download(g, f, ibuf) bind(c, name="plbm_download")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: g
         real(c_double), intent(inout) :: f(*)
         integer(c_int), value :: ibuf
      end function
      integer(c_int) function plbm_stream(g) bind(c, name="plbm_stream")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
      end function
      integer(c_int) function plbm_collide(g) bind(c, name="plbm_collide")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
      end function
      integer(c_int) function plbm_perform_lbm_step(g, nsteps) bind(c, name="plbm_perform_lbm_step")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
         integer(c_int), value :: nsteps
      end function
      integer(c_int) function plbm_update_macros(g, rho, ux, uy) bind(c, name="plbm_update_macros")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: g
         real(c_double), intent(inout) :: rho(*), ux(*), uy(*)
      end function
      type(c_ptr) function plbm_last_error() bind(c, name="plbm_last_error")
         import :: c_ptr
      end function
      integer(c_int) function plbm_set_streaming(g, scheme) bind(c, name="plbm_set_streaming")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
         integer(c_int), value :: scheme
      end function
      integer(c_int) function plbm_set_time_step(g, dt) bind(c, name="plbm_set_time_step")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: g
         real(c_double), value :: dt
      end function
      integer(c_int) function plbm_grid_set_indices3(g, iold, inew, imid) bind(c, name="plbm_grid_set_indices3")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
         integer(c_int), value :: iold, inew, imid
      end function
      integer(c_int) function plbm_perform_triple_step(g, nsteps) bind(c, name="plbm_perform_triple_step")
         import :: c_int, c_ptr
         type(c_ptr), value :: g
         integer(c_int), value :: nsteps
      end function
      integer(c_int) function plbm_output_npy_step(g, folder, filename, step) bind(c, name="plbm_output_npy_step")
         import :: c_int, c_ptr, c_char
         type(c_ptr), value :: g
         character(kind=c_char), intent(in) :: folder(*), filename(*)
         integer(c_int), value :: step
      end function
   end interface

   type :: grid_entry
      integer(c_intptr_t) :: key = 0
      type(c_ptr) :: handle = c_null_ptr
   end type
   integer, parameter :: max_grids = 64
   type(grid_entry), save :: table(max_grids)

contains

   subroutine check(status, what)
      integer(c_int), intent(in) :: status
      character(*), intent(in) :: what
      character(kind=c_char), pointer :: msg(:)
      character(len=512) :: text
      integer :: i
      if (status == 0) return
      call c_f_pointer(plbm_last_error(), msg, [512])
      text = ' '
      do i = 1, 512
         if (msg(i) == char(0)) exit
         text(i:i) = msg(i)
      end do
      write(*,'(a,": ",a)') what, trim(text)
      error stop "plbm_gpu: library error"
   end subroutine

   integer(c_intptr_t) function key_of(grid)
      class(lattice_grid), intent(in), target :: grid
      key_of = transfer(c_loc(grid%f), key_of)
   end function

   type(c_ptr) function handle_of(grid)
      class(lattice_grid), intent(in), target :: grid
      integer :: i
      integer(c_intptr_t) :: k
      k = key_of(grid)
      do i = 1, max_grids
         if (table(i)%key == k) then
            handle_of = table(i)%handle
            return
         end if
      end do
      error stop "plbm_gpu: grid not attached (call plbm_gpu_attach first)"
   end function

   !> Create the device mirror of grid (all nf lattices uploaded).
   subroutine plbm_gpu_attach(grid, math)
      class(lattice_grid), intent(inout), target :: grid
      integer(c_int), intent(in), optional :: math
      type(c_ptr) :: h
      integer :: i, slot
      slot = 0
      do i = 1, max_grids
         if (table(i)%key == 0) then
            slot = i
            exit
         end if
      end do
      if (slot == 0) error stop "plbm_gpu: too many attached grids"
      call check(plbm_grid_create(int(grid%nx, c_int), int(grid%ny, c_int), int(size(grid%f, 4), c_int), &
                                  PLBM_F64, h), "plbm_grid_create")
      table(slot)%key = key_of(grid)
      table(slot)%handle = h
      if (present(math)) call check(plbm_set_math(h, math), "plbm_set_math")
      call plbm_gpu_upload(grid)
   end subroutine

   subroutine plbm_gpu_detach(grid)
      class(lattice_grid), intent(inout), target :: grid
      integer :: i
      integer(c_intptr_t) :: k
      k = key_of(grid)
      do i = 1, max_grids
         if (table(i)%key == k) then
            call check(plbm_grid_destroy(table(i)%handle), "plbm_grid_destroy")
            table(i)%key = 0
            table(i)%handle = c_null_ptr
         end if
      end do
   end subroutine

   !> Host grid%f(:,:,:,b) -> device, every buffer b.
   subroutine plbm_gpu_upload(grid)
      class(lattice_grid), intent(inout), target :: grid
      integer :: b
      do b = 1, size(grid%f, 4)
         call check(plbm_upload(handle_of(grid), grid%f(:,:,:,b), int(b, c_int)), "plbm_upload")
      end do
   end subroutine

   !> Device -> host grid%f(:,:,:,b), every buffer b.
   subroutine plbm_gpu_download(grid)
      class(lattice_grid), intent(inout), target :: grid
      integer :: b
      do b = 1, size(grid%f, 4)
         call check(plbm_download(handle_of(grid), grid%f(:,:,:,b), int(b, c_int)), "plbm_download")
      end do
   end subroutine

   subroutine sync_state(grid, h, kind)
      class(lattice_grid), intent(in) :: grid
      type(c_ptr), intent(in) :: h
      integer(c_int), intent(in) :: kind
      call check(plbm_grid_set_indices(h, int(grid%iold, c_int), int(grid%inew, c_int)), "plbm_grid_set_indices")
      call check(plbm_set_relaxation(h, real(grid%omega, c_double), real(grid%trt_magic, c_double)), &
                 "plbm_set_relaxation")
      if (kind >= 0) call check(plbm_set_collision(h, kind), "plbm_set_collision")
   end subroutine

   !> streaming_interface: f(:,:,:,iold) -> f(:,:,:,inew) on the device.
   subroutine lbm_stream_gpu(grid)
      class(lattice_grid), intent(inout) :: grid
      type(c_ptr) :: h
      h = handle_of(grid)
      call sync_state(grid, h, -1_c_int)
      call check(plbm_stream(h), "plbm_stream")
   end subroutine

   subroutine stream_scheme(grid, scheme)
      class(lattice_grid), intent(inout) :: grid
      integer(c_int), intent(in) :: scheme
      type(c_ptr) :: h
      h = handle_of(grid)
      call sync_state(grid, h, -1_c_int)
      call check(plbm_set_time_step(h, real(grid%dt, c_double)), "plbm_set_time_step")
      call check(plbm_set_streaming(h, scheme), "plbm_set_streaming")
      call check(plbm_stream(h), "plbm_stream")
      call check(plbm_set_streaming(h, 0_c_int), "plbm_set_streaming")
   end subroutine

   !> streaming_interface: stream_fvm_bardow on the device (grid%dt).
   subroutine stream_fvm_bardow_gpu(grid)
      class(lattice_grid), intent(inout) :: grid
      call stream_scheme(grid, 1_c_int)
   end subroutine

   !> streaming_interface: stream_fdm_bardow (central differences) on the device.
   subroutine stream_fdm_bardow_gpu(grid)
      class(lattice_grid), intent(inout) :: grid
      call stream_scheme(grid, 2_c_int)
   end subroutine

   !> streaming_interface: stream_fdm_sofonea on the device.
   subroutine stream_fdm_sofonea_gpu(grid)
      class(lattice_grid), intent(inout) :: grid
      call stream_scheme(grid, 5_c_int)
   end subroutine

   subroutine collide_kind(grid, kind)
      class(lattice_grid), intent(inout) :: grid
      integer(c_int), intent(in) :: kind
      type(c_ptr) :: h
      h = handle_of(grid)
      call sync_state(grid, h, kind)
      call check(plbm_collide(h), "plbm_collide")
   end subroutine

   subroutine collide_bgk_gpu(grid)
      class(lattice_grid), intent(inout) :: grid
      call collide_kind(grid, PLBM_BGK)
   end subroutine

   subroutine collide_trt_gpu(grid)
      class(lattice_grid), intent(inout) :: grid
      call collide_kind(grid, PLBM_TRT)
   end subroutine

   subroutine collide_rr_gpu(grid)
      class(lattice_grid), intent(inout) :: grid
      call collide_kind(grid, PLBM_RR)
   end subroutine

   subroutine collide_bgk_improved_gpu(grid)
      class(lattice_grid), intent(inout) :: grid
      call collide_kind(grid, PLBM_BGKI)
   end subroutine

   !> perform_lbm_step with one fused stream+collide kernel.  The collision
   !> is the one named by kind (default: BGK); the iold/inew swap is the
   !> reference's (src/periodic_lbm.f90:22-27).
   subroutine perform_lbm_step_gpu(grid, kind)
      class(lattice_grid), intent(inout) :: grid
      integer(c_int), intent(in), optional :: kind
      type(c_ptr) :: h
      integer :: itmp
      integer(c_int) :: k
      k = PLBM_BGK
      if (present(kind)) k = kind
      h = handle_of(grid)
      call sync_state(grid, h, k)
      call check(plbm_perform_lbm_step(h, 1_c_int), "plbm_perform_lbm_step")
      itmp = grid%iold
      grid%iold = grid%inew
      grid%inew = itmp
   end subroutine

   !> perform_triple_step with one fused kernel (the pre-collision populations
   !> land in f(:,:,:,iold) of the device state, as in the reference); the
   !> index rotation is the reference's (src/fvm_bardow.F90:333-338).
   subroutine perform_triple_step_gpu(grid, kind)
      class(lattice_grid), intent(inout) :: grid
      integer(c_int), intent(in), optional :: kind
      type(c_ptr) :: h
      integer :: itmp
      integer(c_int) :: k
      k = PLBM_BGK
      if (present(kind)) k = kind
      h = handle_of(grid)
      call sync_state(grid, h, k)
      call check(plbm_grid_set_indices3(h, int(grid%iold, c_int), int(grid%inew, c_int), int(grid%imid, c_int)), &
                 "plbm_grid_set_indices3")
      call check(plbm_perform_triple_step(h, 1_c_int), "plbm_perform_triple_step")
      itmp = grid%iold
      grid%iold = grid%inew
      grid%inew = grid%imid
      grid%imid = itmp
   end subroutine

   !> output_npy: grid%foldername/grid%filename + step (I0.9) + '.npy' holding
   !> mf(ny,nx,3) of the device state's f(:,:,:,inew).
   subroutine output_npy_gpu(grid, step)
      class(lattice_grid), intent(in) :: grid
      integer, intent(in), optional :: step
      type(c_ptr) :: h
      integer(c_int) :: s
      character(len=:), allocatable :: folder
      s = -1
      if (present(step)) s = int(step, c_int)
      folder = ''
      if (allocated(grid%foldername)) folder = trim(grid%foldername)
      h = handle_of(grid)
      call sync_state(grid, h, -1_c_int)
      call check(plbm_output_npy_step(h, folder//c_null_char, grid%filename//c_null_char, s), "plbm_output_npy_step")
   end subroutine

   !> update_macros: moments of f(:,:,:,inew) into grid%rho, grid%ux, grid%uy.
   subroutine update_macros_gpu(grid)
      class(lattice_grid), intent(inout) :: grid
      type(c_ptr) :: h
      h = handle_of(grid)
      call sync_state(grid, h, -1_c_int)
      call check(plbm_update_macros(h, grid%mf(:,:,1), grid%mf(:,:,2), grid%mf(:,:,3)), "plbm_update_macros")
   end subroutine

end module plbm_gpu
