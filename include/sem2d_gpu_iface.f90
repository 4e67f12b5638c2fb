! sem2d_gpu_iface.f90 -- Fortran 2003 ISO_C_BINDING interface to the
! C-ABI of include/sem2d_gpu.h, for SEM2DPACK's own driver.
!
! The derived types repeat the C structures member for member, in the
! header's order (tests/test_abi.py checks names, order and kinds against
! the header and the offsets against the compiled library).  Pointer
! members are type(c_ptr): the driver sets them with c_loc() of its arrays
! (ibool, coord, hprime, ... exactly as init_main leaves them, Fortran
! order, 1-based node numbers) or c_null_ptr.  Every pointer argument of
! the functions is passed by value as type(c_ptr) (c_loc(x) or c_null_ptr),
! handles are type(c_ptr).
!
! Seam in the reference (see INTEGRATION.md for the driver changes):
!   main.f90:54        call solve(pb)  ->  sem2d_gpu_step(h, 1)
!   solver.f90:140-161 solve_leapfrog  ->  the GPU step kernels
!   a non-zero status  ->  call IO_abort(sem2d_error_message(h))
!                          (stdio.f90:205-213)
module sem2d_gpu_iface
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: SEM2D_GPU_ABI_VERSION = 1
  integer(c_int), parameter :: SEM2D_OK = 0
  integer(c_int), parameter :: SEM2D_E_ARG = -1
  integer(c_int), parameter :: SEM2D_E_CUDA = -2
  integer(c_int), parameter :: SEM2D_E_UNSUPPORTED = -3
  integer(c_int), parameter :: SEM2D_E_NR = -4
  integer(c_int), parameter :: SEM2D_E_NAN = -5
  integer(c_int), parameter :: SEM2D_E_STATE = -6
  integer(c_int), parameter :: SEM2D_E_NOMEM = -7
  integer(c_int), parameter :: SEM2D_E_TIMEOUT = -8
  integer(c_int), parameter :: SEM2D_TIME_LEAPFROG = 0
  integer(c_int), parameter :: SEM2D_TIME_NEWMARK = 1
  integer(c_int), parameter :: SEM2D_TIME_HHT = 2
  integer(c_int), parameter :: SEM2D_FRICTION_SWF = 1
  integer(c_int), parameter :: SEM2D_FRICTION_RSF = 2
  integer(c_int), parameter :: SEM2D_FRICTION_TWF = 3
  integer(c_int), parameter :: SEM2D_PRECISION_FP64 = 0
  integer(c_int), parameter :: SEM2D_PRECISION_MIXED = 1
  integer(c_int), parameter :: SEM2D_STF_NONE = 0
  integer(c_int), parameter :: SEM2D_STF_RICKER = 1
  integer(c_int), parameter :: SEM2D_STF_TAB = 3
  integer(c_int), parameter :: SEM2D_STF_HARMONIC = 4
  integer(c_int), parameter :: SEM2D_STF_BRUNE = 5
  integer(c_int), parameter :: SEM2D_STF_GAUSSIAN = 6
  integer(c_int), parameter :: SEM2D_STF_USER = 7
  integer(c_int), parameter :: SEM2D_WAVE_NONE = 0
  integer(c_int), parameter :: SEM2D_WAVE_P = 1
  integer(c_int), parameter :: SEM2D_WAVE_S = 2
  integer(c_int), parameter :: SEM2D_NOALLOC_SCRATCH_BYTES = 8388608

  ! a source time function (STF_get, stf_gen.f90:99-121)
  type, bind(C) :: sem2d_stf
    integer(c_int)         :: kind
    integer(c_int)         :: ntab
    real(c_double)         :: f0
    real(c_double)         :: onset
    real(c_double)         :: ampli
    real(c_double)         :: par1
    real(c_double)         :: par2
    type(c_ptr)            :: tab_t
    type(c_ptr)            :: tab_v
  end type sem2d_stf

  type, bind(C) :: sem2d_problem_desc
    integer(c_int)         :: ngll
    integer(c_int)         :: ndof
    integer(c_int)         :: nelem
    integer(c_int)         :: npoin
    type(c_ptr)            :: ibool
    type(c_ptr)            :: coord
    type(c_ptr)            :: hprime
    type(c_ptr)            :: wgll
    type(c_ptr)            :: Kx
    type(c_ptr)            :: Kz
    type(c_ptr)            :: la
    type(c_ptr)            :: mu
    type(c_ptr)            :: mux
    type(c_ptr)            :: kv_eta
    integer(c_int)         :: kd2_form
    type(c_ptr)            :: rmass
    integer(c_int)         :: nabs
    type(c_ptr)            :: abs_node
    type(c_ptr)            :: abs_C
    integer(c_int)         :: time_scheme
    real(c_double)         :: dt
    real(c_double)         :: beta
    real(c_double)         :: gamma
    integer(c_int)         :: nt
    integer(c_int)         :: nsrc
    type(c_ptr)            :: src_node
    type(c_ptr)            :: src_dir
    type(c_ptr)            :: src_f0
    type(c_ptr)            :: src_t0
    type(c_ptr)            :: src_ampli
    type(c_ptr)            :: src_relamp
    type(c_ptr)            :: src_tdelay
    integer(c_int)         :: nrec
    character(kind=c_char) :: rec_field
    integer(c_int)         :: rec_isamp
    integer(c_int)         :: rec_nsamp
    type(c_ptr)            :: rec_node
    type(c_ptr)            :: rec_elem
    type(c_ptr)            :: rec_interp
    integer(c_int)         :: nflt
    type(c_ptr)            :: flt_node1
    type(c_ptr)            :: flt_node2
    type(c_ptr)            :: flt_n1
    type(c_ptr)            :: flt_B
    type(c_ptr)            :: flt_invM1
    type(c_ptr)            :: flt_invM2
    type(c_ptr)            :: flt_Z
    type(c_ptr)            :: flt_T0
    type(c_ptr)            :: flt_cohesion
    real(c_double)         :: flt_coefA2V
    real(c_double)         :: flt_coefA2D
    integer(c_int)         :: flt_opening
    integer(c_int)         :: flt_friction
    integer(c_int)         :: swf_kind
    integer(c_int)         :: swf_healing
    type(c_ptr)            :: swf_dc
    type(c_ptr)            :: swf_mus
    type(c_ptr)            :: swf_mud
    type(c_ptr)            :: swf_p
    type(c_ptr)            :: swf_alpha
    integer(c_int)         :: rsf_kind
    type(c_ptr)            :: rsf_dc
    type(c_ptr)            :: rsf_mus
    type(c_ptr)            :: rsf_a
    type(c_ptr)            :: rsf_b
    type(c_ptr)            :: rsf_vstar
    type(c_ptr)            :: rsf_vc
    type(c_ptr)            :: rsf_theta
    type(c_ptr)            :: flt_V0
    integer(c_int)         :: normal_kind
    real(c_double)         :: normal_T
    real(c_double)         :: normal_L
    real(c_double)         :: normal_V
    integer(c_int)         :: flt_oit
    integer(c_int)         :: flt_oitd
    integer(c_int)         :: flt_oix1
    integer(c_int)         :: flt_oixn
    integer(c_int)         :: flt_oixd
    integer(c_int)         :: flt_nsamp
    integer(c_int)         :: precision
    real(c_double)         :: width
    integer(c_int)         :: twf_kind
    real(c_double)         :: twf_mus
    real(c_double)         :: twf_mud
    real(c_double)         :: twf_mu0
    real(c_double)         :: twf_X
    real(c_double)         :: twf_Z
    real(c_double)         :: twf_V
    real(c_double)         :: twf_L
    real(c_double)         :: twf_T
    real(c_double)         :: twf_Dc
    type(c_ptr)            :: rho
    integer(c_int)         :: adjoint
    integer(c_int)         :: flt_potency
    integer(c_int)         :: nstacey
    type(c_ptr)            :: stacey_node
    type(c_ptr)            :: stacey_k
    type(c_ptr)            :: stacey_edge
    type(c_ptr)            :: stacey_K
    integer(c_int)         :: ndir
    type(c_ptr)            :: dir_node
    type(c_ptr)            :: dir_comp
    type(c_ptr)            :: dir_after_fault
    real(c_double)         :: alpha
    integer(c_int)         :: nperio
    type(c_ptr)            :: perio_master
    type(c_ptr)            :: perio_slave
    integer(c_int)         :: flt_nr_maxit
    integer(c_int)         :: info_every
    type(c_ptr)            :: src_stf
    integer(c_int)         :: wave_phase
    real(c_double)         :: wave_angle
    real(c_double)         :: wave_ref(2)
    real(c_double)         :: wave_cp
    real(c_double)         :: wave_cs
    real(c_double)         :: wave_mu
    real(c_double)         :: wave_lambda
    real(c_double)         :: wave_tdelay
    type(c_ptr)            :: wave_stf
    type(c_ptr)            :: abs_B
    type(c_ptr)            :: abs_n
    type(c_ptr)            :: abs_wave
    integer(c_int)         :: nneu
    type(c_ptr)            :: neu_node
    type(c_ptr)            :: neu_comp
    type(c_ptr)            :: neu_B
    type(c_ptr)            :: neu_stf
    integer(c_int)         :: nneu_stf
    type(c_ptr)            :: neu_stfs
    type(c_ptr)            :: xjaci
    type(c_ptr)            :: dvol
  end type sem2d_problem_desc

  type, bind(C) :: sem2d_lattice_args
    integer(c_int)         :: ngll
    integer(c_int)         :: ndof
    integer(c_int)         :: precision
    integer(c_int)         :: nx
    integer(c_int)         :: nz
    integer(c_int)         :: LX
    integer(c_int)         :: LZ
    integer(c_int)         :: pitch
    type(c_ptr)            :: row0
    type(c_ptr)            :: hprime
    type(c_ptr)            :: wgll
    type(c_ptr)            :: d
    type(c_ptr)            :: v
    type(c_ptr)            :: rmass
    type(c_ptr)            :: per_rm
    type(c_ptr)            :: per_Ca
    type(c_ptr)            :: per_Cb
    integer(c_int)         :: mat_iso
    type(c_ptr)            :: mat(4)
    type(c_ptr)            :: xix
    type(c_ptr)            :: etaz
    type(c_ptr)            :: dxdxi
    type(c_ptr)            :: dzdeta
    integer(c_int)         :: nsrc
    type(c_ptr)            :: src_I
    type(c_ptr)            :: src_J
    type(c_ptr)            :: src_amp
    integer(c_int)         :: nt
    integer(c_int)         :: step0
    real(c_double)         :: dt
    integer(c_int)         :: kd2_form
    type(c_ptr)            :: status
  end type sem2d_lattice_args

  interface
    function sem2d_gpu_version() bind(C, name="sem2d_gpu_version")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_version
    end function sem2d_gpu_version
    function sem2d_gpu_device_count() bind(C, name="sem2d_gpu_device_count")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_device_count
    end function sem2d_gpu_device_count
    function sem2d_gpu_create(desc, out) bind(C, name="sem2d_gpu_create")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_create
      type(sem2d_problem_desc), intent(in) :: desc
      type(c_ptr), intent(out) :: out
    end function sem2d_gpu_create
    function sem2d_gpu_create_batch(descs, nsim, out) bind(C, name="sem2d_gpu_create_batch")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_create_batch
      type(sem2d_problem_desc), intent(in) :: descs(*)
      integer(c_int), value :: nsim
      type(c_ptr), intent(out) :: out
    end function sem2d_gpu_create_batch
    function sem2d_gpu_batch_open(out) bind(C, name="sem2d_gpu_batch_open")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_batch_open
      type(c_ptr), intent(out) :: out
    end function sem2d_gpu_batch_open
    function sem2d_gpu_batch_add(h, desc) bind(C, name="sem2d_gpu_batch_add")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_batch_add
      type(c_ptr), value :: h
      type(sem2d_problem_desc), intent(in) :: desc
    end function sem2d_gpu_batch_add
    function sem2d_gpu_batch_add_many(h, descs, n) bind(C, name="sem2d_gpu_batch_add_many")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_batch_add_many
      type(c_ptr), value :: h
      type(sem2d_problem_desc), intent(in) :: descs(*)
      integer(c_int), value :: n
    end function sem2d_gpu_batch_add_many
    function sem2d_gpu_batch_close(h) bind(C, name="sem2d_gpu_batch_close")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_batch_close
      type(c_ptr), value :: h
    end function sem2d_gpu_batch_close
    function sem2d_gpu_batch_size(h) bind(C, name="sem2d_gpu_batch_size")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_batch_size
      type(c_ptr), value :: h
    end function sem2d_gpu_batch_size
    function sem2d_gpu_batch_member(h, i) bind(C, name="sem2d_gpu_batch_member")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      type(c_ptr) :: sem2d_gpu_batch_member
      type(c_ptr), value :: h
      integer(c_int), value :: i
    end function sem2d_gpu_batch_member
    function sem2d_gpu_checkpoint_every(h, every) bind(C, name="sem2d_gpu_checkpoint_every")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_checkpoint_every
      type(c_ptr), value :: h
      integer(c_int), value :: every
    end function sem2d_gpu_checkpoint_every
    function sem2d_gpu_adjoint(h, resid, grad_rho, grad_vp, grad_vs) bind(C, name="sem2d_gpu_adjoint")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_adjoint
      type(c_ptr), value :: h
      type(c_ptr), value :: resid
      type(c_ptr), value :: grad_rho
      type(c_ptr), value :: grad_vp
      type(c_ptr), value :: grad_vs
    end function sem2d_gpu_adjoint
    function sem2d_gpu_step(h, nsteps) bind(C, name="sem2d_gpu_step")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_step
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function sem2d_gpu_step
    function sem2d_gpu_step_timed(h, nsteps, ms) bind(C, name="sem2d_gpu_step_timed")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_step_timed
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
      type(c_ptr), value :: ms
    end function sem2d_gpu_step_timed
    function sem2d_gpu_stream(h) bind(C, name="sem2d_gpu_stream")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      type(c_ptr) :: sem2d_gpu_stream
      type(c_ptr), value :: h
    end function sem2d_gpu_stream
    function sem2d_gpu_sync(h) bind(C, name="sem2d_gpu_sync")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_sync
      type(c_ptr), value :: h
    end function sem2d_gpu_sync
    function sem2d_gpu_current_step(h) bind(C, name="sem2d_gpu_current_step")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_current_step
      type(c_ptr), value :: h
    end function sem2d_gpu_current_step
    function sem2d_gpu_get_fields(h, displ, veloc, accel) bind(C, name="sem2d_gpu_get_fields")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_get_fields
      type(c_ptr), value :: h
      type(c_ptr), value :: displ
      type(c_ptr), value :: veloc
      type(c_ptr), value :: accel
    end function sem2d_gpu_get_fields
    function sem2d_gpu_get_seismograms(h, sis) bind(C, name="sem2d_gpu_get_seismograms")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_get_seismograms
      type(c_ptr), value :: h
      type(c_ptr), value :: sis
    end function sem2d_gpu_get_seismograms
    function sem2d_gpu_get_fault(h, out) bind(C, name="sem2d_gpu_get_fault")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_get_fault
      type(c_ptr), value :: h
      type(c_ptr), value :: out
    end function sem2d_gpu_get_fault
    function sem2d_gpu_get_fault_potency(h, out) bind(C, name="sem2d_gpu_get_fault_potency")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_get_fault_potency
      type(c_ptr), value :: h
      type(c_ptr), value :: out
    end function sem2d_gpu_get_fault_potency
    function sem2d_gpu_get_strain_stress(h, strain, stress) bind(C, name="sem2d_gpu_get_strain_stress")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_get_strain_stress
      type(c_ptr), value :: h
      type(c_ptr), value :: strain
      type(c_ptr), value :: stress
    end function sem2d_gpu_get_strain_stress
    function sem2d_gpu_get_info(h, step, vmax, dmax) bind(C, name="sem2d_gpu_get_info")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_get_info
      type(c_ptr), value :: h
      type(c_ptr), value :: step
      type(c_ptr), value :: vmax
      type(c_ptr), value :: dmax
    end function sem2d_gpu_get_info
    function sem2d_gpu_get_fault_state(h, D, V, T, MU, theta) bind(C, name="sem2d_gpu_get_fault_state")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_get_fault_state
      type(c_ptr), value :: h
      type(c_ptr), value :: D
      type(c_ptr), value :: V
      type(c_ptr), value :: T
      type(c_ptr), value :: MU
      type(c_ptr), value :: theta
    end function sem2d_gpu_get_fault_state
    function sem2d_gpu_reset(h) bind(C, name="sem2d_gpu_reset")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_reset
      type(c_ptr), value :: h
    end function sem2d_gpu_reset
    function sem2d_gpu_kernel_launches(h) bind(C, name="sem2d_gpu_kernel_launches")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_long_long) :: sem2d_gpu_kernel_launches
      type(c_ptr), value :: h
    end function sem2d_gpu_kernel_launches
    function sem2d_gpu_tile_shape(h, tx, tz) bind(C, name="sem2d_gpu_tile_shape")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_tile_shape
      type(c_ptr), value :: h
      type(c_ptr), value :: tx
      type(c_ptr), value :: tz
    end function sem2d_gpu_tile_shape
    function sem2d_gpu_destroy(h) bind(C, name="sem2d_gpu_destroy")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_destroy
      type(c_ptr), value :: h
    end function sem2d_gpu_destroy
    function sem2d_gpu_last_error(h) bind(C, name="sem2d_gpu_last_error")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      type(c_ptr) :: sem2d_gpu_last_error
      type(c_ptr), value :: h
    end function sem2d_gpu_last_error
    function sem2d_gpu_step_noalloc(a, nsteps, stream) bind(C, name="sem2d_gpu_step_noalloc")
      import :: c_int, c_double, c_long_long, c_ptr, sem2d_problem_desc, sem2d_lattice_args
      integer(c_int) :: sem2d_gpu_step_noalloc
      type(sem2d_lattice_args), intent(in) :: a
      integer(c_int), value :: nsteps
      type(c_ptr), value :: stream
    end function sem2d_gpu_step_noalloc
    function c_strlen(s) bind(C, name="strlen")
      import :: c_ptr, c_size_t
      integer(c_size_t) :: c_strlen
      type(c_ptr), value :: s
    end function c_strlen
  end interface

contains

  ! the message of sem2d_gpu_last_error(h) as a Fortran string
  function sem2d_error_message(h) result(msg)
    type(c_ptr), intent(in) :: h
    character(len=:), allocatable :: msg
    type(c_ptr) :: p
    character(kind=c_char), pointer :: chars(:)
    integer :: n, k
    p = sem2d_gpu_last_error(h)
    if (.not. c_associated(p)) then
      msg = ''
      return
    end if
    n = int(c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: msg)
    do k = 1, n
      msg(k:k) = chars(k)
    end do
  end function sem2d_error_message

end module sem2d_gpu_iface
