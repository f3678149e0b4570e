! bromoc_gpu_mod.f90 -- Fortran 2003 interface (ISO_C_BINDING) to the C ABI
! of include/bromoc_gpu.h, for cg-gcmc-bd's Fortran driver (simul1.f90).
!
! Every interface below binds one extern "C" entry point of the header with
! the same argument order; every derived type mirrors one parameter struct
! field for field.  Conventions:
!   - a context, batch or adjoint handle is type(c_ptr), passed by value;
!   - C scalars passed by value carry the VALUE attribute; uint32_t and
!     uint64_t arguments travel as integer(c_int32_t) / integer(c_int64_t)
!     with the same bits;
!   - C pointers to arrays are assumed-size dummies (x(*)), passed by
!     reference, so the module arrays of grandmod/gsbpmod go straight in;
!   - pointer fields of the parameter structs are type(c_ptr): set them with
!     c_loc() of TARGET arrays that live until the set_* call returns (the
!     library copies them);
!   - status: every function returns BROMOC_OK (0) or an error code; the
!     message comes from bromoc_gpu_last_error (a C string, see
!     bromoc_error_message below).
module bromoc_gpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: BROMOC_OK = 0, BROMOC_E_ARG = 1, &
       BROMOC_E_STATE = 2, BROMOC_E_CUDA = 3, BROMOC_E_CAPACITY = 4, &
       BROMOC_E_NOMEM = 5, BROMOC_E_DEVICE = 6
  integer(c_int32_t), parameter :: BROMOC_M_NONBOND = 1, BROMOC_M_MEMB = 2, &
       BROMOC_M_PHIX = 4, BROMOC_M_PHIV = 8, BROMOC_M_RFPAR = 16, BROMOC_M_BOND = 32, &
       BROMOC_M_MMIJ = 64, BROMOC_M_ALL = 127
  integer(c_int32_t), parameter :: BROMOC_BOX = 0, BROMOC_SPHERE = 1, BROMOC_ECYL = 2
  integer(c_int32_t), parameter :: BROMOC_FP64 = 0, BROMOC_FP32 = 1
  integer(c_int32_t), parameter :: BROMOC_DYN0 = 0, BROMOC_DYN1 = 1, &
       BROMOC_DYN2 = 2, BROMOC_DYN3 = 3
  ! energy term slots of eterms(1:BROMOC_NTERMS): ener, eelec, evdw, esrpmf,
  ! eefpot, eqqmx, evdwmx, esrpmfmx, eefpotmx, ememb, egsbpa, egsbpb, evdwgd,
  ! erfpar, ebond, eang, edihe, estack, ebp, eex, eqq, esolv, econ
  ! (1-based here: slot k of the header is eterms(k+1))
  integer(c_int32_t), parameter :: BROMOC_NTERMS = 23

  type, bind(C) :: bromoc_system
    integer(c_int32_t) :: shape
    integer(c_int32_t) :: qcountion
    real(c_double) :: lx, ly, lz
    real(c_double) :: cx, cy, cz
    real(c_double) :: rsphe
    real(c_double) :: temp
    real(c_double) :: kbt
    real(c_double) :: cdie
    real(c_double) :: dt
    real(c_double) :: bdmax
  end type bromoc_system

  type, bind(C) :: bromoc_types
    integer(c_int32_t) :: ntype
    integer(c_int32_t) :: nold
    integer(c_int32_t) :: nttyp
    integer(c_int32_t) :: ndna
    type(c_ptr) :: nwtype
    type(c_ptr) :: cg
    type(c_ptr) :: diffusion
  end type bromoc_types

  type, bind(C) :: bromoc_pairs
    integer(c_int32_t) :: ntc
    type(c_ptr) :: qchr, qlj, qsrpmf, qefpot
    type(c_ptr) :: fct
    type(c_ptr) :: epp4
    type(c_ptr) :: sgp2
    type(c_ptr) :: c0, c1, c2, c3, c4
    real(c_double) :: rth
    real(c_double) :: srpx, srpk, srpy
    integer(c_int32_t) :: cnt
    type(c_ptr) :: ep
    type(c_ptr) :: sc
    type(c_ptr) :: dm2
    type(c_ptr) :: dmi
    type(c_ptr) :: nxi
    real(c_double) :: res
  end type bromoc_pairs

  type, bind(C) :: bromoc_sites
    integer(c_int32_t) :: nsites
    type(c_ptr) :: typtyp
    type(c_ptr) :: charge
    type(c_ptr) :: stfree
    type(c_ptr) :: phiv_map
  end type bromoc_sites

  ! nucleotmod's term lists; site lists are term-major (sitebond(2,nbond) on
  ! the Fortran side, i.e. transpose(sitebond(1:nbond,1:2)))
  type, bind(C) :: bromoc_nucleotides
    real(c_double) :: epsnuc
    real(c_double) :: scalepairing
    real(c_double) :: fctn
    real(c_double) :: kappa
    integer(c_int32_t) :: qdeby
    integer(c_int32_t) :: qsolv
    real(c_double) :: epsolv
    integer(c_int32_t) :: nbond
    type(c_ptr) :: sitebond
    type(c_ptr) :: distbond
    integer(c_int32_t) :: nangle
    type(c_ptr) :: siteangle
    type(c_ptr) :: valangle
    integer(c_int32_t) :: ndihe
    type(c_ptr) :: sitedihe
    type(c_ptr) :: valdihe
    integer(c_int32_t) :: nstack
    type(c_ptr) :: sitestack
    type(c_ptr) :: sgstack
    integer(c_int32_t) :: nbp
    type(c_ptr) :: sitebp
    type(c_ptr) :: sgbp
    type(c_ptr) :: bpgc
    integer(c_int32_t) :: nex
    type(c_ptr) :: siteex
    type(c_ptr) :: sgex
    integer(c_int32_t) :: nqq
    type(c_ptr) :: siteqq
    integer(c_int32_t) :: nsolv
    type(c_ptr) :: siteslv
    integer(c_int32_t) :: afn
    type(c_ptr) :: sn
    type(c_ptr) :: af
    integer(c_int32_t) :: ctn
    type(c_ptr) :: csn
    type(c_ptr) :: kx
    type(c_ptr) :: ky
    type(c_ptr) :: kz
    type(c_ptr) :: contrx
    type(c_ptr) :: contry
    type(c_ptr) :: contrz
    integer(c_int32_t) :: qunsplit
    integer(c_int32_t) :: nsites1st
    integer(c_int32_t) :: qnotr(3)
    real(c_double) :: notr(3)
  end type bromoc_nucleotides

  ! gsbpmod's MMIJ basis: RECTBOX orders and region, or SPHERE nmpol/srdist
  type, bind(C) :: bromoc_mmij
    integer(c_int32_t) :: shape
    integer(c_int32_t) :: xnpol, ynpol, znpol
    type(c_ptr) :: lstpx, lstpy, lstpz
    real(c_double) :: rbxmin, rbxmax, rbymin, rbymax, rbzmin, rbzmax
    real(c_double) :: rfscal
    integer(c_int32_t) :: nmpol
    real(c_double) :: srdist
    type(c_ptr) :: mmij
  end type bromoc_mmij

  type, bind(C) :: bromoc_grid
    integer(c_int32_t) :: nclx, ncly, nclz
    real(c_double) :: dcel
    real(c_double) :: xbcen, ybcen, zbcen
  end type bromoc_grid

  type, bind(C) :: bromoc_phiv_opts
    integer(c_int32_t) :: nmaps
    integer(c_int32_t) :: trilinear
    integer(c_int32_t) :: nmcden
    real(c_double) :: svdw, vzmin, vzmax, thold8, thold27
    type(c_ptr) :: map_of_type
    type(c_ptr) :: scal
  end type bromoc_phiv_opts

  type, bind(C) :: bromoc_membrane
    integer(c_int32_t) :: qpore
    real(c_double) :: voltage
    real(c_double) :: afact, ikappa, ceps, zmemb1, zmemb2
    type(c_ptr) :: ampl1
    type(c_ptr) :: p1
    type(c_ptr) :: ampl2
    type(c_ptr) :: p2
    type(c_ptr) :: rcylinder
  end type bromoc_membrane

  type, bind(C) :: bromoc_diffusion
    real(c_double) :: plength2, pcenter
    type(c_ptr) :: ampl3
    type(c_ptr) :: p3
    integer(c_int32_t) :: nspline
    type(c_ptr) :: xs, ys, b, c, d
    real(c_double) :: diff0, ibeta, diffcutoff
    real(c_double) :: fact0n1, fact0n2
    integer(c_int32_t) :: qdnafree
  end type bromoc_diffusion

  type, bind(C) :: bromoc_buffers
    integer(c_int32_t) :: nbuffer
    type(c_ptr) :: ibfftyp
    type(c_ptr) :: avnum, mu, kb, lzmin, lzmax, rmin, rmax
    type(c_ptr) :: qbufferbias
    type(c_ptr) :: nat
    type(c_ptr) :: ntotat
  end type bromoc_buffers

  interface
    ! ---- context ----------------------------------------------------------
    function bromoc_gpu_create(capacity, precision, stream, ctx) &
         bind(C, name="bromoc_gpu_create") result(rc)
      import :: c_int, c_int32_t, c_ptr
      integer(c_int32_t), value :: capacity, precision
      type(c_ptr), value :: stream
      type(c_ptr), intent(out) :: ctx
      integer(c_int) :: rc
    end function
    function bromoc_gpu_destroy(ctx) bind(C, name="bromoc_gpu_destroy") result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int) :: rc
    end function
    function bromoc_gpu_last_error(ctx) bind(C, name="bromoc_gpu_last_error") result(msg)
      import :: c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr) :: msg
    end function
    function bromoc_gpu_abi_version() bind(C, name="bromoc_gpu_abi_version") result(v)
      import :: c_int
      integer(c_int) :: v
    end function

    ! ---- module state (deck-time fills) -----------------------------------
    function bromoc_gpu_set_system(ctx, sys) bind(C, name="bromoc_gpu_set_system") result(rc)
      import :: c_int, c_ptr, bromoc_system
      type(c_ptr), value :: ctx
      type(bromoc_system), intent(in) :: sys
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_types(ctx, t) bind(C, name="bromoc_gpu_set_types") result(rc)
      import :: c_int, c_ptr, bromoc_types
      type(c_ptr), value :: ctx
      type(bromoc_types), intent(in) :: t
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_pairs(ctx, p) bind(C, name="bromoc_gpu_set_pairs") result(rc)
      import :: c_int, c_ptr, bromoc_pairs
      type(c_ptr), value :: ctx
      type(bromoc_pairs), intent(in) :: p
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_sites(ctx, s) bind(C, name="bromoc_gpu_set_sites") result(rc)
      import :: c_int, c_ptr, bromoc_sites
      type(c_ptr), value :: ctx
      type(bromoc_sites), intent(in) :: s
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_nucleotides(ctx, nuc) bind(C, name="bromoc_gpu_set_nucleotides") &
         result(rc)
      import :: c_int, c_ptr, bromoc_nucleotides
      type(c_ptr), value :: ctx
      type(bromoc_nucleotides), intent(in) :: nuc
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_mmij(ctx, m) bind(C, name="bromoc_gpu_set_mmij") result(rc)
      import :: c_int, c_ptr, bromoc_mmij
      type(c_ptr), value :: ctx
      type(bromoc_mmij), intent(in) :: m
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_phix(ctx, g, phix) bind(C, name="bromoc_gpu_set_phix") result(rc)
      import :: c_int, c_ptr, c_float, bromoc_grid
      type(c_ptr), value :: ctx
      type(bromoc_grid), intent(in) :: g
      real(c_float), intent(in) :: phix(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_phiv(ctx, g, phiv, opts) bind(C, name="bromoc_gpu_set_phiv") result(rc)
      import :: c_int, c_ptr, c_int8_t, bromoc_grid, bromoc_phiv_opts
      type(c_ptr), value :: ctx
      type(bromoc_grid), intent(in) :: g
      integer(c_int8_t), intent(in) :: phiv(*)
      type(bromoc_phiv_opts), intent(in) :: opts
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_rfpar(ctx, g, nmaps, gsrfen, greff, reffac, map_of_type) &
         bind(C, name="bromoc_gpu_set_rfpar") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_float, c_double, bromoc_grid
      type(c_ptr), value :: ctx
      type(bromoc_grid), intent(in) :: g
      integer(c_int32_t), value :: nmaps
      real(c_float), intent(in) :: gsrfen(*), greff(*)
      real(c_double), value :: reffac
      integer(c_int32_t), intent(in) :: map_of_type(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_membrane(ctx, m) bind(C, name="bromoc_gpu_set_membrane") result(rc)
      import :: c_int, c_ptr, bromoc_membrane
      type(c_ptr), value :: ctx
      type(bromoc_membrane), intent(in) :: m
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_diffusion(ctx, d) bind(C, name="bromoc_gpu_set_diffusion") result(rc)
      import :: c_int, c_ptr, bromoc_diffusion
      type(c_ptr), value :: ctx
      type(bromoc_diffusion), intent(in) :: d
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_countions(ctx, cntpts, zcont) &
         bind(C, name="bromoc_gpu_set_countions") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: cntpts
      real(c_double), intent(in) :: zcont(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_buffers(ctx, b) bind(C, name="bromoc_gpu_set_buffers") result(rc)
      import :: c_int, c_ptr, bromoc_buffers
      type(c_ptr), value :: ctx
      type(bromoc_buffers), intent(in) :: b
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_periodic(ctx, on, rcut) bind(C, name="bromoc_gpu_set_periodic") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: on
      real(c_double), value :: rcut
      integer(c_int) :: rc
    end function

    ! ---- particles --------------------------------------------------------
    function bromoc_gpu_set_particles(ctx, ntot, nsites, nfix, x, y, z, typei, ibuffer) &
         bind(C, name="bromoc_gpu_set_particles") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: ntot, nsites, nfix
      real(c_double), intent(in) :: x(*), y(*), z(*)
      integer(c_int32_t), intent(in) :: typei(*), ibuffer(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_get_particles(ctx, ntot, x, y, z, typei, ibuffer) &
         bind(C, name="bromoc_gpu_get_particles") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(out) :: ntot
      real(c_double), intent(out) :: x(*), y(*), z(*)
      integer(c_int32_t), intent(out) :: typei(*), ibuffer(*)
      integer(c_int) :: rc
    end function

    ! ---- hot path: ENERGY, INTERACT, DYNAMICS, BD loop, GRAND ---------------
    function bromoc_gpu_energy(ctx, terms, qforces, fx, fy, fz, eterms, warn) &
         bind(C, name="bromoc_gpu_energy") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: terms, qforces
      real(c_double), intent(out) :: fx(*), fy(*), fz(*), eterms(*)
      integer(c_int32_t), intent(out) :: warn(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_interact(ctx, terms, xj, yj, zj, jtype, j, dener) &
         bind(C, name="bromoc_gpu_interact") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: terms
      real(c_double), value :: xj, yj, zj
      integer(c_int32_t), value :: jtype, j
      real(c_double), intent(out) :: dener
      integer(c_int) :: rc
    end function
    function bromoc_gpu_dynamics(ctx, variant, seed, step) &
         bind(C, name="bromoc_gpu_dynamics") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: variant
      integer(c_int64_t), value :: seed, step
      integer(c_int) :: rc
    end function
    function bromoc_gpu_bd_steps(ctx, terms, variant, nsteps, seed, step0, eterms) &
         bind(C, name="bromoc_gpu_bd_steps") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: terms, variant, nsteps
      integer(c_int64_t), value :: seed, step0
      real(c_double), intent(out) :: eterms(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_bd_steps_host(ctx, terms, variant, nsteps, seed, step0, ntot, &
         nsites, nfix, x, y, z, typei, eterms) &
         bind(C, name="bromoc_gpu_bd_steps_host") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: terms, variant, nsteps
      integer(c_int64_t), value :: seed, step0
      integer(c_int32_t), value :: ntot, nsites, nfix
      real(c_double), intent(inout) :: x(*), y(*), z(*)
      integer(c_int32_t), intent(in) :: typei(*)
      real(c_double), intent(out) :: eterms(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_simul_cycles_host(ctx, terms, variant, ncycle, ngcmc, nbd, seed, &
         cycle0, ntot, nsites, nfix, x, y, z, typei, ibuffer, eterms) &
         bind(C, name="bromoc_gpu_simul_cycles_host") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: terms, variant, ncycle, ngcmc, nbd
      integer(c_int64_t), value :: seed, cycle0
      integer(c_int32_t), intent(inout) :: ntot
      integer(c_int32_t), value :: nsites, nfix
      real(c_double), intent(inout) :: x(*), y(*), z(*)
      integer(c_int32_t), intent(inout) :: typei(*), ibuffer(*)
      real(c_double), intent(out) :: eterms(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_grand(ctx, terms, ngcmc, seed, cycle, dener_sum) &
         bind(C, name="bromoc_gpu_grand") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: terms, ngcmc
      integer(c_int64_t), value :: seed, cycle
      real(c_double), intent(out) :: dener_sum
      integer(c_int) :: rc
    end function
    function bromoc_gpu_get_buffers(ctx, nat, ninsert, nremove, prob) &
         bind(C, name="bromoc_gpu_get_buffers") result(rc)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(out) :: nat(*), ninsert(*), nremove(*), prob(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_get_countions(ctx, nforward, nbackward) &
         bind(C, name="bromoc_gpu_get_countions") result(rc)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(out) :: nforward(*), nbackward(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_get_dids(ctx, dids) bind(C, name="bromoc_gpu_get_dids") result(rc)
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: dids(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_count(ctx) bind(C, name="bromoc_gpu_count") result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int) :: rc
    end function
    function bromoc_gpu_get_ntotat(ctx, ntotat) bind(C, name="bromoc_gpu_get_ntotat") result(rc)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(out) :: ntotat(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_profiles(ctx, qrho, qrdna, qgr, igr, dr, npoints) &
         bind(C, name="bromoc_gpu_set_profiles") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: qrho, qrdna, qgr, igr
      real(c_double), value :: dr
      integer(c_int32_t), value :: npoints
      integer(c_int) :: rc
    end function
    function bromoc_gpu_accum_profiles(ctx) bind(C, name="bromoc_gpu_accum_profiles") result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int) :: rc
    end function
    function bromoc_gpu_get_profiles(ctx, rho, rdna, gr, nzmax, irmax) &
         bind(C, name="bromoc_gpu_get_profiles") result(rc)
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: rho(*), rdna(*), gr(*)
      integer(c_int32_t), intent(out) :: nzmax, irmax
      integer(c_int) :: rc
    end function
    function bromoc_gpu_traj_header(nframe, nttyp, atnam, buf, cap, nbytes) &
         bind(C, name="bromoc_gpu_traj_header") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_char
      integer(c_int32_t), value :: nframe, nttyp
      character(kind=c_char), intent(in) :: atnam(*)
      type(c_ptr), value :: buf
      integer(c_int64_t), value :: cap
      integer(c_int64_t), intent(out) :: nbytes
      integer(c_int) :: rc
    end function
    function bromoc_gpu_traj_frame(ctx, runtime, buf, cap, nbytes) &
         bind(C, name="bromoc_gpu_traj_frame") result(rc)
      import :: c_int, c_ptr, c_double, c_int64_t
      type(c_ptr), value :: ctx
      real(c_double), value :: runtime
      type(c_ptr), value :: buf
      integer(c_int64_t), value :: cap
      integer(c_int64_t), intent(out) :: nbytes
      integer(c_int) :: rc
    end function
    function bromoc_gpu_efpot_from_knots(n, xx, yy, fct, qchr, ep, sc3, dm2o, dmio) &
         bind(C, name="bromoc_gpu_efpot_from_knots") result(rc)
      import :: c_int, c_int32_t, c_double
      integer(c_int32_t), value :: n
      real(c_double), intent(in) :: xx(*), yy(*)
      real(c_double), value :: fct
      integer(c_int32_t), value :: qchr
      real(c_double), intent(out) :: ep(*), sc3(*), dm2o(*), dmio(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_pair_energy_static(ctx, n, nfix, x, y, z, typei, fx, fy, fz, &
         eterms4) bind(C, name="bromoc_gpu_pair_energy_static") result(rc)
      ! device buffers (a CUDA Fortran or OpenACC caller passes device
      ! addresses); declared c_ptr here
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: n, nfix
      type(c_ptr), value :: x, y, z, typei, fx, fy, fz, eterms4
      integer(c_int) :: rc
    end function
    function bromoc_gpu_live_count_async(ctx, dst) &
         bind(C, name="bromoc_gpu_live_count_async") result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: dst
      integer(c_int) :: rc
    end function
    function bromoc_gpu_set_fused_bd(ctx, on) bind(C, name="bromoc_gpu_set_fused_bd") result(rc)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: on
      integer(c_int) :: rc
    end function

    function bromoc_gpu_metropolis(ctx, terms, nmcm, mcmax, seed, cycle, naccept, dener_sum) &
         bind(C, name="bromoc_gpu_metropolis") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: terms, nmcm
      real(c_double), value :: mcmax
      integer(c_int64_t), value :: seed, cycle
      integer(c_int32_t), intent(out) :: naccept
      real(c_double), intent(out) :: dener_sum
      integer(c_int) :: rc
    end function

    ! ---- measurement hooks and self-tests ----------------------------------
    function bromoc_gpu_kernel_timing(ctx, on) bind(C, name="bromoc_gpu_kernel_timing") result(rc)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: on
      integer(c_int) :: rc
    end function
    function bromoc_gpu_kernel_time(ctx, which, total_ms, launches) &
         bind(C, name="bromoc_gpu_kernel_time") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: which
      real(c_double), intent(out) :: total_ms
      integer(c_int64_t), intent(out) :: launches
      integer(c_int) :: rc
    end function
    function bromoc_gpu_launch_count(ctx) bind(C, name="bromoc_gpu_launch_count") result(n)
      import :: c_ptr, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int64_t) :: n
    end function
    function bromoc_gpu_fp32_peak(stream, tflops) bind(C, name="bromoc_gpu_fp32_peak") result(rc)
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: stream
      real(c_double), intent(out) :: tflops
      integer(c_int) :: rc
    end function
    function bromoc_gpu_ff_check(fn, n, x, out) bind(C, name="bromoc_gpu_ff_check") result(rc)
      import :: c_int, c_int32_t, c_double
      integer(c_int32_t), value :: fn, n
      real(c_double), intent(in) :: x(*)
      real(c_double), intent(out) :: out(*)
      integer(c_int) :: rc
    end function
    function bromoc_gpu_wait_selftest(spins, arrive, err_word) &
         bind(C, name="bromoc_gpu_wait_selftest") result(rc)
      import :: c_int, c_int32_t
      integer(c_int32_t), value :: spins, arrive
      integer(c_int32_t), intent(out) :: err_word
      integer(c_int) :: rc
    end function

    ! ---- replica batches ----------------------------------------------------
    function bromoc_batch_create(proto, nrep, capacity, b) &
         bind(C, name="bromoc_batch_create") result(rc)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: proto
      integer(c_int32_t), value :: nrep
      integer(c_int32_t), intent(in) :: capacity(*)
      type(c_ptr), intent(out) :: b
      integer(c_int) :: rc
    end function
    function bromoc_batch_destroy(b) bind(C, name="bromoc_batch_destroy") result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int) :: rc
    end function
    function bromoc_batch_set_systems(b, sys) bind(C, name="bromoc_batch_set_systems") result(rc)
      import :: c_int, c_ptr, bromoc_system
      type(c_ptr), value :: b
      type(bromoc_system), intent(in) :: sys(*)
      integer(c_int) :: rc
    end function
    function bromoc_batch_set_particles(b, r, n, x, y, z, typei) &
         bind(C, name="bromoc_batch_set_particles") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: b
      integer(c_int32_t), value :: r, n
      real(c_double), intent(in) :: x(*), y(*), z(*)
      integer(c_int32_t), intent(in) :: typei(*)
      integer(c_int) :: rc
    end function
    function bromoc_batch_get_particles(b, r, n, x, y, z) &
         bind(C, name="bromoc_batch_get_particles") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: b
      integer(c_int32_t), value :: r
      integer(c_int32_t), intent(out) :: n
      real(c_double), intent(out) :: x(*), y(*), z(*)
      integer(c_int) :: rc
    end function
    function bromoc_batch_bd_steps(b, terms, nsteps, seeds, step0, eterms) &
         bind(C, name="bromoc_batch_bd_steps") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
      type(c_ptr), value :: b
      integer(c_int32_t), value :: terms, nsteps
      integer(c_int64_t), intent(in) :: seeds(*)
      integer(c_int64_t), value :: step0
      real(c_double), intent(out) :: eterms(*)
      integer(c_int) :: rc
    end function
    function bromoc_batch_energy(b, terms, forces, eterms) &
         bind(C, name="bromoc_batch_energy") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: b
      integer(c_int32_t), value :: terms
      real(c_double), intent(out) :: forces(*), eterms(*)
      integer(c_int) :: rc
    end function
    function bromoc_batch_offset(b, r) bind(C, name="bromoc_batch_offset") result(off)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: b
      integer(c_int32_t), value :: r
      integer(c_int) :: off
    end function

    function bromoc_batch_last_error(b) bind(C, name="bromoc_batch_last_error") result(msg)
      import :: c_ptr
      type(c_ptr), value :: b
      type(c_ptr) :: msg
    end function
    function bromoc_batch_slots(b) bind(C, name="bromoc_batch_slots") result(n)
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int) :: n
    end function
    function bromoc_batch_set_graph(b, on) bind(C, name="bromoc_batch_set_graph") result(rc)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: b
      integer(c_int32_t), value :: on
      integer(c_int) :: rc
    end function
    function bromoc_batch_tuning(b, warps, items, ms) bind(C, name="bromoc_batch_tuning") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: b
      integer(c_int32_t), intent(out) :: warps(*), items(*)
      real(c_double), intent(out) :: ms(*)
      integer(c_int) :: rc
    end function
    function bromoc_batch_graph_launches(b) bind(C, name="bromoc_batch_graph_launches") result(n)
      import :: c_ptr, c_int64_t
      type(c_ptr), value :: b
      integer(c_int64_t) :: n
    end function
    function bromoc_batch_launch_count(b) bind(C, name="bromoc_batch_launch_count") result(n)
      import :: c_ptr, c_int64_t
      type(c_ptr), value :: b
      integer(c_int64_t) :: n
    end function
    function bromoc_batch_set_buffers(b, r, buf, ibuffer) &
         bind(C, name="bromoc_batch_set_buffers") result(rc)
      import :: c_int, c_ptr, c_int32_t, bromoc_buffers
      type(c_ptr), value :: b
      integer(c_int32_t), value :: r
      type(bromoc_buffers), intent(in) :: buf
      integer(c_int32_t), intent(in) :: ibuffer(*)
      integer(c_int) :: rc
    end function
    function bromoc_batch_grand(b, terms, ngcmc, seeds, cycle, dener) &
         bind(C, name="bromoc_batch_grand") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
      type(c_ptr), value :: b
      integer(c_int32_t), value :: terms, ngcmc
      integer(c_int64_t), intent(in) :: seeds(*)
      integer(c_int64_t), value :: cycle
      real(c_double), intent(out) :: dener(*)
      integer(c_int) :: rc
    end function
    function bromoc_batch_count(b) bind(C, name="bromoc_batch_count") result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int) :: rc
    end function
    function bromoc_batch_get_buffers(b, r, nat, ninsert, nremove, typei, ibuffer) &
         bind(C, name="bromoc_batch_get_buffers") result(rc)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: b
      integer(c_int32_t), value :: r
      integer(c_int32_t), intent(out) :: nat(*), ninsert(*), nremove(*), typei(*), ibuffer(*)
      integer(c_int) :: rc
    end function

    ! ---- adjoint of a BD segment ------------------------------------------
    function bromoc_adj_create(proto, capacity, precision, a) &
         bind(C, name="bromoc_adj_create") result(rc)
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: proto
      integer(c_int32_t), value :: capacity, precision
      type(c_ptr), intent(out) :: a
      integer(c_int) :: rc
    end function
    function bromoc_adj_destroy(a) bind(C, name="bromoc_adj_destroy") result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: a
      integer(c_int) :: rc
    end function
    function bromoc_adj_set_particles(a, n, x, y, z, typei) &
         bind(C, name="bromoc_adj_set_particles") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: a
      integer(c_int32_t), value :: n
      real(c_double), intent(in) :: x(*), y(*), z(*)
      integer(c_int32_t), intent(in) :: typei(*)
      integer(c_int) :: rc
    end function
    function bromoc_adj_forward(a, nsteps, ckpt, seed, step0, nbins, r0, dr, sigma, hist) &
         bind(C, name="bromoc_adj_forward") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
      type(c_ptr), value :: a
      integer(c_int32_t), value :: nsteps, ckpt
      integer(c_int64_t), value :: seed, step0
      integer(c_int32_t), value :: nbins
      real(c_double), value :: r0, dr, sigma
      real(c_double), intent(out) :: hist(*)
      integer(c_int) :: rc
    end function
    function bromoc_adj_backward(a, dl_dhist, g_ep, g_sc) &
         bind(C, name="bromoc_adj_backward") result(rc)
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: a
      real(c_double), intent(in) :: dl_dhist(*)
      real(c_double), intent(out) :: g_ep(*), g_sc(*)
      integer(c_int) :: rc
    end function
    function bromoc_adj_get_particles(a, which, x, y, z) &
         bind(C, name="bromoc_adj_get_particles") result(rc)
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: a
      integer(c_int32_t), value :: which
      real(c_double), intent(out) :: x(*), y(*), z(*)
      integer(c_int) :: rc
    end function
    function bromoc_adj_last_error(a) bind(C, name="bromoc_adj_last_error") result(msg)
      import :: c_ptr
      type(c_ptr), value :: a
      type(c_ptr) :: msg
    end function
  end interface

  interface
    function bromoc_c_strlen(s) bind(C, name="strlen") result(n)
      import :: c_ptr, c_size_t
      type(c_ptr), value :: s
      integer(c_size_t) :: n
    end function
  end interface

contains

  ! The last error message of a context as a Fortran string.
  function bromoc_error_message(ctx) result(msg)
    type(c_ptr), intent(in) :: ctx
    character(len=:), allocatable :: msg
    type(c_ptr) :: p
    character(kind=c_char), pointer :: chars(:)
    integer :: n, k
    p = bromoc_gpu_last_error(ctx)
    if (.not. c_associated(p)) then
      msg = ''
      return
    end if
    n = int(bromoc_c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: msg)
    do k = 1, n
      msg(k:k) = chars(k)
    end do
  end function bromoc_error_message

end module bromoc_gpu
