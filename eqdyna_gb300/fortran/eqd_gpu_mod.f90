! ISO_C_BINDING interface of libeqdyna_gb300.so (include/eqdyna_gb300.h) for the EQdyna Fortran
! driver.  The derived types mirror the C structs field by field; array fields are C pointers
! obtained with c_loc() on the globalvar arrays, which are passed without copies.
module eqd_gpu_mod
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: EQD_OK = 0, EQD_ERR_NAN = 4
  integer(c_int), parameter :: EQD_PREC_FP64 = 0, EQD_PREC_FP32 = 1
  integer(c_int), parameter :: EQD_TABLES_AUTO = 0, EQD_TABLES_STREAMED = 1, EQD_TABLES_RECORDS = 2

  type, bind(C) :: eqd_scalars
    real(c_double) :: dt, rdampk, rdampm, grav, roumax, rhow, gamar, w, kapa_hg
    real(c_double) :: xsource, ysource, zsource, nucR, nucRuptVel, nucdtau0, nucT
    real(c_double) :: PMLb(8), vmaxPML, R, ccosphi, sinphi, tv, dx, slipRateThres
    real(c_double) :: fric_tp_h, time0
    integer(c_int32_t) :: C_elastic, C_Q, C_hg, friclaw, TPV, C_nuclea, nucfault
    integer(c_int32_t) :: insertFaultType, nPML, nstep, mode, reserved
  end type

  type, bind(C) :: eqd_host_arrays
    integer(c_int32_t) :: nnode, nelem, neq, size_eqidx
    integer(c_int64_t) :: size_stress
    type(c_ptr) :: nodeElemIdRelation, elemTypeArr, eqNumIndexArr, eqNumStartIndexLoc
    type(c_ptr) :: numOfDofPerNodeArr, meshCoor, eleshp, eledet, mat, elemass, ss, phi
    type(c_ptr) :: stressArr, stressCompIndexArr, pstrain, eleporep, nodalMassArr, fnms
    type(c_ptr) :: v1, velArr, dispArr, nodalForceArr
    integer(c_int32_t) :: ntotft, nftmx
    type(c_ptr) :: nftnd, nsmp, un, us, ud, arn, fric, fnft
    integer(c_int32_t) :: numOnFaultSt, numOffFaultSt
    type(c_ptr) :: anonfs, idhist, onFaultQuantHistSCECForm, OffFaultStGramSCEC, onFaultTPHist
  end type

  type, bind(C) :: eqd_options
    integer(c_int32_t) :: precision, learned_guess, record_tp_hist, tile_shape
    integer(c_int32_t) :: use_graph, device, table_layout, block_node, block_fault, sequential_fault
  end type

  ! device addresses of the globalvar arrays for eqd_gpu_elem_forces_noalloc (arrays already on
  ! the GPU under OpenACC or CUDA Fortran; the call allocates nothing)
  type, bind(C) :: eqd_elem_device_view
    integer(c_int32_t) :: nnode, nelem
    type(c_ptr) :: nodeElemIdRelation, elemTypeArr, eleshp, eledet, mat, ss, phi
    type(c_ptr) :: stressArr, stressCompIndexArr, velArr, dispArr
    real(c_double) :: dt, rdampk, w
    integer(c_int64_t) :: size_stress
    integer(c_int32_t) :: C_elastic, C_Q, C_hg
  end type

  interface
    integer(c_int) function eqd_gpu_init(s, a, opt, ctx) bind(C, name="eqd_gpu_init")
      import :: c_int, c_ptr, eqd_scalars, eqd_host_arrays, eqd_options
      type(eqd_scalars), intent(in) :: s
      type(eqd_host_arrays), intent(in) :: a
      type(eqd_options), intent(in) :: opt
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function eqd_gpu_step(ctx, nt_begin, nsteps) bind(C, name="eqd_gpu_step")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: nt_begin, nsteps
    end function
    integer(c_int) function eqd_gpu_fetch(ctx, a) bind(C, name="eqd_gpu_fetch")
      import :: c_int, c_ptr, eqd_host_arrays
      type(c_ptr), value :: ctx
      type(eqd_host_arrays), intent(inout) :: a
    end function
    integer(c_int) function eqd_gpu_fetch_fault(ctx, fric, fnft) bind(C, name="eqd_gpu_fetch_fault")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, fric, fnft
    end function
    integer(c_int) function eqd_gpu_finalize(ctx) bind(C, name="eqd_gpu_finalize")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    type(c_ptr) function eqd_gpu_status_string(status) bind(C, name="eqd_gpu_status_string")
      import :: c_ptr, c_int
      integer(c_int), value :: status
    end function
    ! per-step result reads and the pipelined loop
    integer(c_int) function eqd_gpu_fetch_fric_rows(ctx, rows, nrows, dst) bind(C, name="eqd_gpu_fetch_fric_rows")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx, rows, dst
      integer(c_int32_t), value :: nrows
    end function
    integer(c_int) function eqd_gpu_step_async(ctx, nt_begin, nsteps) bind(C, name="eqd_gpu_step_async")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: nt_begin, nsteps
    end function
    integer(c_int) function eqd_gpu_fetch_fric_rows_async(ctx, rows, nrows, dst, ticket) &
        bind(C, name="eqd_gpu_fetch_fric_rows_async")
      import :: c_int, c_ptr, c_int32_t, c_int64_t
      type(c_ptr), value :: ctx, rows, dst
      integer(c_int32_t), value :: nrows
      integer(c_int64_t), intent(out) :: ticket
    end function
    integer(c_int) function eqd_gpu_fetch_wait(ctx, ticket) bind(C, name="eqd_gpu_fetch_wait")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: ticket
    end function
    type(c_ptr) function eqd_host_alloc(bytes) bind(C, name="eqd_host_alloc")
      import :: c_ptr, c_int64_t
      integer(c_int64_t), value :: bytes
    end function
    integer(c_int) function eqd_host_free(p) bind(C, name="eqd_host_free")
      import :: c_int, c_ptr
      type(c_ptr), value :: p
    end function
    ! setup on the GPU: the tables of assembleGlobalMass from the mesh (any output may be c_null_ptr)
    integer(c_int) function eqd_gpu_element_tables(device, a, eleshp, eledet, elemass, ss, phi, &
        nodalMassArr, fnms) bind(C, name="eqd_gpu_element_tables")
      import :: c_int, c_int32_t, c_ptr, eqd_host_arrays
      integer(c_int32_t), value :: device
      type(eqd_host_arrays), intent(in) :: a
      type(c_ptr), value :: eleshp, eledet, elemass, ss, phi, nodalMassArr, fnms
    end function
    integer(c_int) function eqd_gpu_elem_forces_noalloc(view, force_out, stream) &
        bind(C, name="eqd_gpu_elem_forces_noalloc")
      import :: c_int, c_ptr, eqd_elem_device_view
      type(eqd_elem_device_view), intent(in) :: view
      type(c_ptr), value :: force_out, stream
    end function
  end interface

contains

  ! Fills the two argument structs from module globalvar (all arrays must be allocated and
  ! carry the TARGET attribute, or be passed through a TARGET dummy, for c_loc).
  subroutine eqd_fill_from_globalvar(s, a)
    use globalvar
    type(eqd_scalars), intent(out) :: s
    type(eqd_host_arrays), intent(out) :: a
    s%dt = dt; s%rdampk = rdampk; s%rdampm = rdampm; s%grav = grav; s%roumax = roumax
    s%rhow = rhow; s%gamar = gamar; s%w = w; s%kapa_hg = kapa_hg
    s%xsource = xsource; s%ysource = ysource; s%zsource = zsource; s%nucR = nucR
    s%nucRuptVel = nucRuptVel; s%nucdtau0 = nucdtau0; s%nucT = nucT
    s%PMLb = PMLb; s%vmaxPML = vmaxPML; s%R = R; s%ccosphi = ccosphi; s%sinphi = sinphi
    s%tv = tv; s%dx = dx; s%slipRateThres = slipRateThres; s%fric_tp_h = fric_tp_h
    s%time0 = timeElapsed
    s%C_elastic = C_elastic; s%C_Q = C_Q; s%C_hg = C_hg; s%friclaw = friclaw; s%TPV = TPV
    s%C_nuclea = C_nuclea; s%nucfault = nucfault; s%insertFaultType = insertFaultType
    s%nPML = nPML; s%nstep = nstep; s%mode = mode; s%reserved = 0
    a%nnode = totalNumOfNodes; a%nelem = totalNumOfElements; a%neq = totalNumOfEquations
    a%size_eqidx = sizeOfEqNumIndexArr; a%size_stress = size(stressArr, kind=c_int64_t)
    a%nodeElemIdRelation = c_loc(nodeElemIdRelation); a%elemTypeArr = c_loc(elemTypeArr)
    a%eqNumIndexArr = c_loc(eqNumIndexArr); a%eqNumStartIndexLoc = c_loc(eqNumStartIndexLoc)
    a%numOfDofPerNodeArr = c_loc(numOfDofPerNodeArr); a%meshCoor = c_loc(meshCoor)
    a%eleshp = c_loc(eleshp); a%eledet = c_loc(eledet); a%mat = c_loc(mat)
    a%elemass = c_loc(elemass); a%ss = c_loc(ss); a%phi = c_loc(phi)
    a%stressArr = c_loc(stressArr); a%stressCompIndexArr = c_loc(stressCompIndexArr)
    a%pstrain = c_loc(pstrain); a%eleporep = c_loc(eleporep)
    a%nodalMassArr = c_loc(nodalMassArr); a%fnms = c_loc(fnms); a%v1 = c_loc(v1)
    a%velArr = c_loc(velArr); a%dispArr = c_loc(dispArr); a%nodalForceArr = c_loc(nodalForceArr)
    a%ntotft = ntotft; a%nftmx = nftmx; a%nftnd = c_loc(nftnd); a%nsmp = c_loc(nsmp)
    a%un = c_loc(un); a%us = c_loc(us); a%ud = c_loc(ud); a%arn = c_loc(arn)
    a%fric = c_loc(fric); a%fnft = c_loc(fnft)
    a%numOnFaultSt = numOfOnFaultStCount; a%numOffFaultSt = numOfOffFaultStCount
    a%anonfs = c_loc(anonfs); a%onFaultQuantHistSCECForm = c_loc(onFaultQuantHistSCECForm)
    a%onFaultTPHist = c_loc(onFaultTPHist)
    a%idhist = c_null_ptr; a%OffFaultStGramSCEC = c_null_ptr
    if (numOfOffFaultStCount > 0) then
      a%idhist = c_loc(idhist); a%OffFaultStGramSCEC = c_loc(OffFaultStGramSCEC)
    endif
  end subroutine

end module eqd_gpu_mod
