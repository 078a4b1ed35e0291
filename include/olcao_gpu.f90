! ISO_C_BINDING interface of libolcao_gb300 (include/olcao_gpu.h) for the
! Fortran host code of OLCAO (src/olcao).  The derived types mirror the C
! structures field for field; every procedure binds one C entry point.  A
! maintainer adds this module to the OLCAOsetup / OLCAOmain builds and links
! libolcao_gb300.so; the procedures it replaces are listed in INTEGRATION.md.
!
! Arrays are passed in Fortran (column-major) order, as the C side expects.
! Status 0 means success; gb300Check turns any other status into the
! reference's behaviour at its stop sites (message to unit 20, stop).

module O_GB300
   use iso_c_binding
   implicit none

   ! olc_op_t
   integer(c_int), parameter :: OLC_OP_OVERLAP = 1, OLC_OP_KINETIC = 2, OLC_OP_NUCLEAR = 3, &
         & OLC_OP_ELECPOT = 4, OLC_OP_MASSVEL = 5, OLC_OP_HAMILTONIAN = 6
   ! olc_precision_t, olc_form_t, iteration flags
   integer(c_int), parameter :: OLC_PREC_FP64 = 0, OLC_PREC_MIXED = 1
   integer(c_int), parameter :: OLC_FORM_FUSED = 0, OLC_FORM_STORED = 1
   integer(c_int), parameter :: OLC_ITER_EIG_DEVICE = 1, OLC_ITER_COEFF_DEVICE = 2, &
         & OLC_ITER_GRAPH = 4

   type, bind(C) :: olc_atom_type_t
      integer(c_int32_t) :: element
      integer(c_int32_t) :: num_orb_alphas(4)
      real(c_double)     :: alphas(32)
      integer(c_int32_t) :: num_vale_radial, num_core_radial
      integer(c_int32_t) :: radial_l(12)
      real(c_double)     :: radial_coeff(32, 12)   ! C [12][32] = Fortran (32,12)
   end type

   type, bind(C) :: olc_pot_type_t
      integer(c_int32_t) :: element, num_alphas
      real(c_double)     :: nuc_charge, nuc_alpha
      real(c_double)     :: alphas(32)
   end type

   type, bind(C) :: olc_system_t
      real(c_double)     :: real_vectors(9)
      integer(c_int32_t) :: num_atom_types
      type(c_ptr)        :: atom_types
      integer(c_int32_t) :: num_atom_sites
      type(c_ptr)        :: site_type, site_pos
      integer(c_int32_t) :: num_pot_types
      type(c_ptr)        :: pot_types
      integer(c_int32_t) :: num_pot_sites
      type(c_ptr)        :: pot_site_type, pot_site_pos
      integer(c_int32_t) :: num_kpoints
      type(c_ptr)        :: kpoints_abc
      real(c_double)     :: basis_fn_thresh
      integer(c_int32_t) :: rel              ! O_Potential's rel (1: mass velocity in H)
   end type

   type, bind(C) :: olc_dims_t
      integer(c_int32_t) :: vale_dim, core_dim, pot_dim, num_kpoints
      integer(c_int32_t) :: num_cells, num_pair_tasks
      integer(c_int64_t) :: packed_len
   end type

   type(c_ptr), save :: gb300Ctx = c_null_ptr

   interface
      integer(c_int) function olc_create(sys, stream, ctx) bind(C, name="olc_create")
         import :: c_int, c_ptr, olc_system_t
         type(olc_system_t), intent(in) :: sys
         type(c_ptr), value :: stream
         type(c_ptr), intent(out) :: ctx
      end function
      integer(c_int) function olc_destroy(ctx) bind(C, name="olc_destroy")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
      end function
      integer(c_int) function olc_get_dims(ctx, dims) bind(C, name="olc_get_dims")
         import :: c_int, c_ptr, olc_dims_t
         type(c_ptr), value :: ctx
         type(olc_dims_t), intent(out) :: dims
      end function
      integer(c_int) function olc_last_error(buf, len) bind(C, name="olc_last_error")
         import :: c_int, c_char, c_size_t
         character(kind=c_char), intent(out) :: buf(*)
         integer(c_size_t), value :: len
      end function

      ! gaussOverlapOL/KE/MV/NP, elecPotGaussOverlap (integrals.F90:81-2598):
      ! device arrays valeVale(valeDim,valeDim,nk), coreVale(coreDim,valeDim,nk),
      ! coreCore(coreDim,coreDim,nk) of complex(double)
      integer(c_int) function olc_gauss_overlap(ctx, op, term, coeffs, precision, vv, cv, cc) &
            & bind(C, name="olc_gauss_overlap")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx, coeffs, vv, cv, cc
         integer(c_int), value :: op, term, precision
      end function
      ! ortho(opCode) / orthoOL with packing (integrals.F90:2601-2853)
      integer(c_int) function olc_ortho_pack(ctx, isOverlap, vv, cv, cc, scv, packed) &
            & bind(C, name="olc_ortho_pack")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx, vv, cv, cc, scv, packed
         integer(c_int), value :: isOverlap
      end function
      ! readPackedMatrixAccum loop of secularEqn.F90:128-166 (device arrays)
      integer(c_int) function olc_assemble_hamiltonian(ctx, terms, coeffs, nterm, packedH) &
            & bind(C, name="olc_assemble_hamiltonian")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx, terms, packedH
         real(c_double), intent(in) :: coeffs(*)
         integer(c_int), value :: nterm
      end function
      ! solveZHEGV (interfaces.F90:73-120) for every k at once
      integer(c_int) function olc_solve_zhegv(ctx, packedH, packedS, numStates, eigenValues, &
            & vectors, info) bind(C, name="olc_solve_zhegv")
         import :: c_int, c_ptr, c_double, c_int32_t
         type(c_ptr), value :: ctx, packedH, packedS, vectors
         integer(c_int), value :: numStates
         real(c_double), intent(out) :: eigenValues(*)
         integer(c_int32_t), intent(out) :: info(*)
      end function

      ! setupSCF's integral passes, kept resident (OLCAO_Setup.f90:127-192)
      integer(c_int) function olc_scf_prepare(ctx, precision, form) bind(C, name="olc_scf_prepare")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int), value :: precision, form
      end function
      ! secularEqnAllKP (secularEqn.F90:33-287)
      integer(c_int) function olc_scf_iteration(ctx, coeffs, precision, numStates, &
            & eigenValues, flags, vectors) bind(C, name="olc_scf_iteration")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double), intent(in) :: coeffs(*)
         integer(c_int), value :: precision, numStates, flags
         real(c_double), intent(out) :: eigenValues(*)
         type(c_ptr), value :: vectors
      end function
      ! unpackMatrix of one k (matrixSubs.F90:314-355), host destination
      integer(c_int) function olc_scf_matrices(ctx, coeffs, kpoint, h, s, onDevice) &
            & bind(C, name="olc_scf_matrices")
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: ctx
         real(c_double), intent(in) :: coeffs(*)
         integer(c_int), value :: kpoint, onDevice
         complex(c_double_complex), intent(out) :: h(*), s(*)
      end function

      ! populateStates (populate.F90:132-578)
      integer(c_int) function olc_populate_states(numStates, numKPoints, spin, eigenValues, &
            & kPointWeight, numElectrons, thermalSigma, fermiSearchLimit, maxThermalRange, &
            & population, occupiedEnergy) bind(C, name="olc_populate_states")
         import :: c_int, c_double
         integer(c_int), value :: numStates, numKPoints, spin
         real(c_double), intent(in) :: eigenValues(*), kPointWeight(*)
         real(c_double), value :: numElectrons, thermalSigma, fermiSearchLimit, maxThermalRange
         real(c_double), intent(out) :: population(*), occupiedEnergy
      end function
      ! makeValenceRho (valeCharge.F90:34-420)
      integer(c_int) function olc_make_valence_rho(ctx, numStates, spin, population, &
            & eigenValues, vectors, traces, electronEnergy, rhoPacked) &
            & bind(C, name="olc_make_valence_rho")
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int), value :: numStates, spin
         real(c_double), intent(in) :: population(*), eigenValues(*)
         type(c_ptr), value :: vectors, rhoPacked
         real(c_double), intent(out) :: traces(*), electronEnergy(*)
      end function

      ! the datasets of setup-temp.hdf5 and main-temp.hdf5 (hdf5SetupIntg.F90,
      ! hdf5MainEvec.F90) as raw files plus a manifest
      integer(c_int) function olc_write_setup_integrals(ctx, root) &
            & bind(C, name="olc_write_setup_integrals")
         import :: c_int, c_ptr, c_char
         type(c_ptr), value :: ctx
         character(kind=c_char), intent(in) :: root(*)
      end function
      integer(c_int) function olc_write_eigen(root, nk, spin, numStates, valeDim, eigenValues, &
            & vectors) bind(C, name="olc_write_eigen")
         import :: c_int, c_char, c_double, c_ptr
         character(kind=c_char), intent(in) :: root(*)
         integer(c_int), value :: nk, spin, numStates, valeDim
         real(c_double), intent(in) :: eigenValues(*)
         type(c_ptr), value :: vectors
      end function

      ! library version string (NUL-terminated, static storage)
      type(c_ptr) function olc_version() bind(C, name="olc_version")
         import :: c_ptr
      end function
      ! work of the context on another CUDA stream (c_null_ptr: legacy stream)
      integer(c_int) function olc_set_stream(ctx, stream) bind(C, name="olc_set_stream")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx, stream
      end function

      ! allocation-free solve for n <= 64 from caller-owned DEVICE arrays:
      ! packedH, packedS (2, n(n+1)/2, nk), eigenValues (numStates, nk),
      ! vectors (n, numStates, nk) or c_null_ptr, info (nk); no counterpart
      ! in the reference (see include/olcao_gpu.h for the limits)
      integer(c_int) function olc_solve_zhegv_noalloc(n, nk, packedH, packedS, numStates, &
            & eigenValues, vectors, info, stream) bind(C, name="olc_solve_zhegv_noalloc")
         import :: c_int, c_ptr
         integer(c_int), value :: n, nk, numStates
         type(c_ptr), value :: packedH, packedS, eigenValues, vectors, info, stream
      end function

      ! the tensor-core products the mixed solver uses, on DEVICE arrays
      ! (column-major): FP64-accurate c = a b and FP32-accurate c = op(a) b
      integer(c_int) function olc_split_zgemm(ctx, m, n, k, a, b, c) bind(C, name="olc_split_zgemm")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx, a, b, c
         integer(c_int), value :: m, n, k
      end function
      integer(c_int) function olc_split_cgemm32(ctx, m, n, k, a, conjA, b, c) &
            & bind(C, name="olc_split_cgemm32")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx, a, b, c
         integer(c_int), value :: m, n, k, conjA
      end function

      ! the generated primitives (gaussIntegrals.f90) for a batch of explicit
      ! inputs: kind 1 overlap, 2 kinetic, 3 nuclear, 4 electron 3-centre,
      ! 5 mass velocity, 6 / 7 / 8 momentum x / y / z; inputs(12, n) =
      ! (a1, a2, a3, A, B, C), lmAlpha(2, n), sh(16, 16, n) (host arrays)
      integer(c_int) function olc_primitive_batch(kind, n, inputs, lmAlpha, sh) &
            & bind(C, name="olc_primitive_batch")
         import :: c_int, c_double, c_int32_t
         integer(c_int), value :: kind, n
         real(c_double), intent(in) :: inputs(*)
         integer(c_int32_t), intent(in) :: lmAlpha(*)
         real(c_double), intent(out) :: sh(*)
      end function

      ! stage timing and work counters (the reference's timeStampStart /
      ! timeStampEnd around its stages), and the library's kernel count
      integer(c_int) function olc_profile_enable(ctx, on) bind(C, name="olc_profile_enable")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int), value :: on
      end function
      integer(c_int) function olc_profile_reset(ctx) bind(C, name="olc_profile_reset")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
      end function
      integer(c_int) function olc_profile_read(ctx, stage, launches, ms) bind(C, name="olc_profile_read")
         import :: c_int, c_ptr, c_int64_t, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: stage
         integer(c_int64_t), intent(out) :: launches
         real(c_double), intent(out) :: ms
      end function
      integer(c_int) function olc_profile_read_work(ctx, stage, flops, bytes) &
            & bind(C, name="olc_profile_read_work")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: stage
         real(c_double), intent(out) :: flops, bytes
      end function
      integer(c_int64_t) function olc_launch_count() bind(C, name="olc_launch_count")
         import :: c_int64_t
      end function
   end interface

contains

   ! The reference stops with a message on unit 20 at its error sites; every
   ! call into the library is wrapped the same way.
   subroutine gb300Check(status, where)
      integer(c_int), intent(in) :: status
      character(len=*), intent(in) :: where
      character(kind=c_char) :: msg(512)
      integer(c_int) :: ok
      integer :: i
      character(len=512) :: text
      if (status /= 0) then
         ok = olc_last_error(msg, 512_c_size_t)      ! NUL-terminated message
         text = ' '
         do i = 1, 512
            if (msg(i) == c_null_char) exit
            text(i:i) = msg(i)
         enddo
         write (20,*) where, ': ', trim(text)
         stop
      endif
   end subroutine gb300Check

   ! Null-terminated copy of a Fortran string for the file-writing entries.
   function gb300CString(s) result(c)
      character(len=*), intent(in) :: s
      character(kind=c_char) :: c(len_trim(s) + 1)
      integer :: i
      do i = 1, len_trim(s)
         c(i) = s(i:i)
      enddo
      c(len_trim(s) + 1) = c_null_char
   end function gb300CString
end module O_GB300
