! FEMSolverGPUClass.f90 -- plantFEM's FEMSolver_ call surface over libpfg.so.
!
! Two modules for a plantFEM program (compile with the plantFEM sources, link
! -lpfg): pfg_capi binds the C ABI of include/pfg.h through ISO_C_BINDING,
! field for field and argument for argument; FEMSolverGPUClass wraps it in a
! type FEMSolverGPU_ whose type-bound procedures carry FEMSolver_'s names,
! arguments and defaults (FEMSolverClass.f90:86-162), so that replacing
!     type(FEMSolver_) :: solver
! by
!     type(FEMSolverGPU_) :: solver
! moves setCRS / setMatrix / fix / solve / eig onto the GPU.  As the
! reference, a failing call prints its message and stops the program.
module pfg_capi
   use iso_c_binding
   implicit none

   integer(c_int32_t), parameter :: PFG_ALG_BICGSTAB = 0, PFG_ALG_CG = 1
   integer(c_int32_t), parameter :: PFG_PREC_FP64 = 0, PFG_PREC_MIXED = 1
   integer(c_int32_t), parameter :: PFG_STORAGE_FULL = 0, PFG_STORAGE_SYMMETRIC = 1
   integer(c_int32_t), parameter :: PFG_PC_NONE = 0, PFG_PC_JACOBI = 1, PFG_PC_BLOCK_JACOBI = 2, &
                                    PFG_PC_ILU0 = 3, PFG_PC_ILU0_SORTED = 4
   integer(c_int32_t), parameter :: PFG_STOP_REFERENCE = 0, PFG_STOP_TRUE_RELATIVE = 1

   ! field for field as include/pfg.h: a shorter type would let the library
   ! write past its end
   type, bind(C) :: pfg_solve_opts
      integer(c_int32_t) :: algorithm, precision, precond, stop_rule, itrmax, graph_chunk
      real(c_double)     :: er0, relative_er, reliable_delta
      integer(c_int32_t) :: debug, update_mode, storage
   end type

   type, bind(C) :: pfg_info
      integer(c_int32_t) :: status, iterations, replacements, kernel_launches
      real(c_double)     :: rel_residual, iter_residual, solve_ms
      integer(c_int32_t) :: fallback
   end type

   type, bind(C) :: pfg_eig_opts
      integer(c_int32_t) :: block_size, max_itr
      real(c_double)     :: tol
      integer(c_int32_t) :: precision, precond, stop_rule, debug
      integer(c_int64_t) :: seed
      real(c_double)     :: tol_fp32
   end type

   interface
      subroutine pfg_solve_opts_default(o) bind(C, name="pfg_solve_opts_default")
         import :: pfg_solve_opts
         type(pfg_solve_opts), intent(out) :: o
      end subroutine
      subroutine pfg_eig_opts_default(o) bind(C, name="pfg_eig_opts_default")
         import :: pfg_eig_opts
         type(pfg_eig_opts), intent(out) :: o
      end subroutine
      type(c_ptr) function pfg_last_error() bind(C, name="pfg_last_error")
         import
      end function
      integer(c_int) function pfg_create(h) bind(C, name="pfg_create")
         import
         type(c_ptr), intent(out) :: h
      end function
      integer(c_int) function pfg_destroy(h) bind(C, name="pfg_destroy")
         import
         type(c_ptr), value :: h
      end function
      integer(c_int) function pfg_set_mesh(h, nn, nodcoord, ne, nne, elemnod) bind(C, name="pfg_set_mesh")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), value :: nn, ne
         integer(c_int32_t), value :: nne
         real(c_double), intent(in) :: nodcoord(*)     ! NodCoord(nn,3), column-major as in Mesh_
         integer(c_int32_t), intent(in) :: elemnod(*)  ! ElemNod(ne,8), 1-based
      end function
      integer(c_int) function pfg_set_crs(h, dof) bind(C, name="pfg_set_crs")
         import
         type(c_ptr), value :: h
         integer(c_int32_t), value :: dof
      end function
      integer(c_int) function pfg_set_crs_arrays(h, n, row_ptr, col_idx, val) bind(C, name="pfg_set_crs_arrays")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), value :: n
         integer(c_int64_t), intent(in) :: row_ptr(*)
         integer(c_int32_t), intent(in) :: col_idx(*)
         real(c_double), intent(in) :: val(*)
      end function
      integer(c_int) function pfg_get_crs_size(h, n, nnz) bind(C, name="pfg_get_crs_size")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), intent(out) :: n, nnz
      end function
      integer(c_int) function pfg_get_crs(h, row_ptr, col_idx, val) bind(C, name="pfg_get_crs")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), intent(out) :: row_ptr(*)
         integer(c_int32_t), intent(out) :: col_idx(*)
         real(c_double), intent(out) :: val(*)
      end function
      integer(c_int) function pfg_set_rhs(h, n, rhs) bind(C, name="pfg_set_rhs")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), value :: n
         real(c_double), intent(in) :: rhs(*)
      end function
      integer(c_int) function pfg_get_rhs(h, n, rhs) bind(C, name="pfg_get_rhs")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), value :: n
         real(c_double), intent(out) :: rhs(*)
      end function
      integer(c_int) function pfg_set_matrix(h, domain_id, element_id, dof, matrix) bind(C, name="pfg_set_matrix")
         import
         type(c_ptr), value :: h
         integer(c_int32_t), value :: domain_id, element_id, dof
         real(c_double), intent(in) :: matrix(*)       ! (nne*dof) x (nne*dof), column-major
      end function
      integer(c_int) function pfg_set_vector(h, domain_id, element_id, dof, vector) bind(C, name="pfg_set_vector")
         import
         type(c_ptr), value :: h
         integer(c_int32_t), value :: domain_id, element_id, dof
         real(c_double), intent(in) :: vector(*)
      end function
      integer(c_int) function pfg_assemble_stiffness(h, n_prop, E, nu) bind(C, name="pfg_assemble_stiffness")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), value :: n_prop
         real(c_double), intent(in) :: E(*), nu(*)
      end function
      integer(c_int) function pfg_assemble_mass(h, n_prop, rho, lumped) bind(C, name="pfg_assemble_mass")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), value :: n_prop
         real(c_double), intent(in) :: rho(*)
         integer(c_int32_t), value :: lumped
      end function
      integer(c_int) function pfg_zeros(h) bind(C, name="pfg_zeros")
         import
         type(c_ptr), value :: h
      end function
      integer(c_int) function pfg_fix(h, n, ids, values, value) bind(C, name="pfg_fix")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), value :: n
         integer(c_int32_t), intent(in) :: ids(*)
         type(c_ptr), value :: values                   ! c_loc(FixValues) or c_null_ptr
         real(c_double), value :: value
      end function
      integer(c_int) function pfg_solve(h, opts, x0, x_out, info) bind(C, name="pfg_solve")
         import
         type(c_ptr), value :: h
         type(pfg_solve_opts), intent(in) :: opts
         type(c_ptr), value :: x0                       ! c_loc(x0) or c_null_ptr
         real(c_double), intent(out) :: x_out(*)
         type(pfg_info), intent(out) :: info
      end function
      integer(c_int) function pfg_keep_this_matrix_as(h, name) bind(C, name="pfg_keep_this_matrix_as")
         import
         type(c_ptr), value :: h
         character(kind=c_char), intent(in) :: name(*)  ! NUL-terminated
      end function
      integer(c_int) function pfg_load_matrix(h, name) bind(C, name="pfg_load_matrix")
         import
         type(c_ptr), value :: h
         character(kind=c_char), intent(in) :: name(*)
      end function
      integer(c_int) function pfg_fix_eig(h, n, ids) bind(C, name="pfg_fix_eig")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), value :: n
         integer(c_int32_t), intent(in) :: ids(*)
      end function
      integer(c_int) function pfg_eig(h, opts, num_eigen, eigen_value, eigen_vectors, info) bind(C, name="pfg_eig")
         import
         type(c_ptr), value :: h
         type(pfg_eig_opts), intent(in) :: opts
         integer(c_int32_t), value :: num_eigen
         real(c_double), intent(out) :: eigen_value(*)
         real(c_double), intent(out) :: eigen_vectors(*)  ! ndof x num_eigen, column-major
         type(pfg_info), intent(out) :: info
      end function
      integer(c_int) function pfg_eig_dense(h, num_eigen, eigen_value, eigen_vectors, info) &
         bind(C, name="pfg_eig_dense")
         import
         type(c_ptr), value :: h
         integer(c_int32_t), value :: num_eigen
         real(c_double), intent(out) :: eigen_value(*)
         real(c_double), intent(out) :: eigen_vectors(*)
         type(pfg_info), intent(out) :: info
      end function
      integer(c_int) function pfg_eig_reduced_size(h, n) bind(C, name="pfg_eig_reduced_size")
         import
         type(c_ptr), value :: h
         integer(c_int64_t), intent(out) :: n
      end function
      integer(c_int) function pfg_element_stress(h, displacement, n_prop, E, v, option, out) &
         bind(C, name="pfg_element_stress")
         import
         type(c_ptr), value :: h
         real(c_double), intent(in) :: displacement(*), E(*), v(*)
         integer(c_int64_t), value :: n_prop
         integer(c_int32_t), value :: option
         real(c_double), intent(out) :: out(*)
      end function
      ! drop-in for crs_spmv_real64 (SparseClass.f90:38-51): the same arguments,
      ! an integer status instead of a subroutine
      integer(c_int) function pfg_crs_spmv_real64(val, row_ptr, col_idx, old_vector, new_vector, n, col_size) &
         bind(C, name="pfg_crs_spmv_real64")
         import
         integer(c_size_t), value :: n, col_size
         real(c_double), intent(in) :: val(*), old_vector(*)
         integer(c_int64_t), intent(in) :: row_ptr(*)
         integer(c_int32_t), intent(in) :: col_idx(*)
         real(c_double), intent(inout) :: new_vector(*)
      end function
      ! the LinearSolver hook of FEMSolver_%solve (FEMSolverClass.f90:1632-1662)
      integer(c_int) function pfg_linear_solver_crs(row_ptr, col_idx, val, rhs, x, n, nnz, opts, info) &
         bind(C, name="pfg_linear_solver_crs")
         import
         integer(c_int64_t), intent(in) :: row_ptr(*)
         integer(c_int32_t), intent(in) :: col_idx(*)
         real(c_double), intent(in) :: val(*), rhs(*)
         real(c_double), intent(inout) :: x(*)
         integer(c_int64_t), value :: n, nnz
         type(pfg_solve_opts), intent(in) :: opts
         type(pfg_info), intent(out) :: info
      end function
   end interface

contains

   ! pfg_last_error() as a Fortran string
   function pfg_error_message() result(msg)
      character(len=:), allocatable :: msg
      character(kind=c_char), pointer :: p(:)
      type(c_ptr) :: cp
      integer :: n
      cp = pfg_last_error()
      msg = ""
      if (.not. c_associated(cp)) return
      call c_f_pointer(cp, p, [4096])
      n = 0
      do while (n < 4096)
         if (p(n + 1) == c_null_char) exit
         n = n + 1
      end do
      allocate (character(len=n) :: msg)
      msg = transfer(p(1:n), msg)
   end function

   ! the reference's error behaviour: print and stop
   subroutine pfg_check(rc, where)
      integer(c_int), intent(in) :: rc
      character(*), intent(in) :: where
      if (rc < 0) then
         print *, "ERROR :: FEMSolverGPU_%"//where//" >> "//pfg_error_message()
         stop
      end if
   end subroutine

end module pfg_capi

module FEMSolverGPUClass
   use iso_fortran_env
   use iso_c_binding
   use pfg_capi
   use FEMDomainClass
   implicit none

   ! FEMSolver_'s public fields and defaults (FEMSolverClass.f90:60-80), the
   ! working matrix read back by getCRS, and the handle of the C ABI
   type :: FEMSolverGPU_
      type(c_ptr) :: handle = c_null_ptr
      integer(int32) :: itrmax = 100000
      real(real64)   :: er0 = dble(1.0e-10)
      real(real64)   :: relative_er = dble(1.0e-10)
      logical        :: debug = .false.
      logical        :: use_LOBPCG = .false.
      integer(int32) :: LOBPCG_MAX_ITR = 100000
      real(real64)   :: LOBPCG_TOL = dble(1.0e-6)
      integer(int32) :: LOBPCG_NUM_MODE = 5
      ! GB300 forms (not in the reference): mixed precision, CG, symmetric storage
      logical        :: mixed_precision = .false.
      logical        :: symmetric_storage = .false.
      real(real64), allocatable :: CRS_val(:), CRS_RHS(:)
      integer(int32), allocatable :: CRS_Index_Col(:)
      integer(int64), allocatable :: CRS_Index_Row(:)
   contains
      procedure, public :: init => initFEMSolverGPU
      procedure, public :: setDomain => setDomainFEMSolverGPU
      procedure, public :: setCRS => setCRSFEMSolverGPU
      procedure, public :: setRHS => setRHSFEMSolverGPU
      procedure, public :: setMatrix => setMatrixFEMSolverGPU
      procedure, public :: setVector => setVectorFEMSolverGPU
      procedure, public :: fix => fixFEMSolverGPU
      procedure, public :: solve => solveFEMSolverGPU
      procedure, public :: zeros => zerosFEMSolverGPU
      procedure, public :: keepThisMatrixAs => keepThisMatrixAsFEMSolverGPU
      procedure, public :: loadMatrix => loadMatrixFEMSolverGPU
      procedure, public :: fix_eig => fix_eigFEMSolverGPU
      procedure, public :: eig => eigFEMSolverGPU
      procedure, public :: getCRS => getCRSFEMSolverGPU
      procedure, public :: remove => removeFEMSolverGPU
   end type

contains

   ! FEMSolver_%init(NumDomain) (FEMSolverClass.f90:174-327): one domain
   subroutine initFEMSolverGPU(this, NumDomain)
      class(FEMSolverGPU_), intent(inout) :: this
      integer(int32), optional, intent(in) :: NumDomain
      if (present(NumDomain)) then
         if (NumDomain /= 1) then
            print *, "ERROR :: FEMSolverGPU_%init >> one domain (overset coupling is not on the GPU path)"
            stop
         end if
      end if
      if (c_associated(this%handle)) call this%remove()
      call pfg_check(pfg_create(this%handle), "init")
   end subroutine

   ! FEMSolver_%setDomain(FEMDomain, DomainID) (FEMSolverClass.f90:329-419)
   subroutine setDomainFEMSolverGPU(this, FEMDomain, DomainID)
      class(FEMSolverGPU_), intent(inout) :: this
      type(FEMDomain_), intent(in) :: FEMDomain
      integer(int32), optional, intent(in) :: DomainID
      if (.not. c_associated(this%handle)) call this%init()
      call pfg_check(pfg_set_mesh(this%handle, int(size(FEMDomain%mesh%nodcoord, 1), c_int64_t), &
                                  FEMDomain%mesh%nodcoord, int(size(FEMDomain%mesh%elemnod, 1), c_int64_t), &
                                  int(size(FEMDomain%mesh%elemnod, 2), c_int32_t), FEMDomain%mesh%elemnod), &
                     "setDomain")
   end subroutine

   ! FEMSolver_%setCRS(DOF) (FEMSolverClass.f90:439-898)
   subroutine setCRSFEMSolverGPU(this, DOF)
      class(FEMSolverGPU_), intent(inout) :: this
      integer(int32), intent(in) :: DOF
      call pfg_check(pfg_set_crs(this%handle, int(DOF, c_int32_t)), "setCRS")
   end subroutine

   ! FEMSolver_%setRHS(RHS) (FEMSolverClass.f90:431-437)
   subroutine setRHSFEMSolverGPU(this, RHS)
      class(FEMSolverGPU_), intent(inout) :: this
      real(real64), intent(in) :: RHS(:)
      call pfg_check(pfg_set_rhs(this%handle, int(size(RHS), c_int64_t), RHS), "setRHS")
   end subroutine

   ! FEMSolver_%setMatrix(DomainID, ElementID, DOF, Matrix) (FEMSolverClass.f90:1020-1057)
   subroutine setMatrixFEMSolverGPU(this, DomainID, ElementID, DOF, Matrix)
      class(FEMSolverGPU_), intent(inout) :: this
      integer(int32), intent(in) :: DomainID, ElementID, DOF
      real(real64), intent(in) :: Matrix(:, :)
      call pfg_check(pfg_set_matrix(this%handle, int(DomainID, c_int32_t), int(ElementID, c_int32_t), &
                                    int(DOF, c_int32_t), Matrix), "setMatrix")
   end subroutine

   ! FEMSolver_%setVector(DomainID, ElementID, DOF, Vector) (FEMSolverClass.f90:913-920)
   subroutine setVectorFEMSolverGPU(this, DomainID, ElementID, DOF, Vector)
      class(FEMSolverGPU_), intent(inout) :: this
      integer(int32), intent(in) :: DomainID, ElementID, DOF
      real(real64), intent(in) :: Vector(:)
      call pfg_check(pfg_set_vector(this%handle, int(DomainID, c_int32_t), int(ElementID, c_int32_t), &
                                    int(DOF, c_int32_t), Vector), "setVector")
   end subroutine

   ! FEMSolver_%fix(DomainID, IDs, FixValue | FixValues) (FEMSolverClass.f90:1073-1136)
   subroutine fixFEMSolverGPU(this, DomainID, IDs, FixValue, FixValues)
      class(FEMSolverGPU_), intent(inout) :: this
      integer(int32), intent(in) :: DomainID
      integer(int32), intent(in) :: IDs(:)
      real(real64), optional, intent(in) :: FixValue
      real(real64), optional, target, intent(in) :: FixValues(:)
      real(c_double) :: v
      type(c_ptr) :: vp
      v = 0.0d0
      if (present(FixValue)) v = FixValue
      vp = c_null_ptr
      if (present(FixValues)) vp = c_loc(FixValues)
      call pfg_check(pfg_fix(this%handle, int(size(IDs), c_int64_t), IDs, vp, v), "fix")
   end subroutine

   ! x = FEMSolver_%solve([algorithm], [preconditioning], [x0]) (FEMSolverClass.f90:1697-1825);
   ! defaults as the reference: FP64 BiCGSTAB, no preconditioner, its stop rule
   function solveFEMSolverGPU(this, algorithm, preconditioning, x0) result(x)
      class(FEMSolverGPU_), intent(inout) :: this
      character(*), optional, intent(in) :: algorithm, preconditioning
      real(real64), optional, target, intent(in) :: x0(:)
      real(real64), allocatable :: x(:)
      type(pfg_solve_opts) :: o
      type(pfg_info) :: info
      integer(c_int64_t) :: n, nnz
      type(c_ptr) :: xp
      call pfg_solve_opts_default(o)
      o%itrmax = this%itrmax
      o%er0 = this%er0
      o%relative_er = this%relative_er
      o%debug = merge(1, 0, this%debug)
      if (present(algorithm)) then
         if (algorithm == "CG") o%algorithm = PFG_ALG_CG
      end if
      if (present(preconditioning)) then
         select case (preconditioning)
         case ("Jacobi", "PointJacobi")
            o%precond = PFG_PC_JACOBI
         case ("BlockJacobi")
            o%precond = PFG_PC_BLOCK_JACOBI
         case ("ILU", "incompleteLU")
            o%precond = PFG_PC_ILU0
         end select
      end if
      if (this%mixed_precision) then
         o%precision = PFG_PREC_MIXED
         o%stop_rule = PFG_STOP_TRUE_RELATIVE
         if (this%symmetric_storage) o%storage = PFG_STORAGE_SYMMETRIC
      end if
      call pfg_check(pfg_get_crs_size(this%handle, n, nnz), "solve")
      allocate (x(n))
      xp = c_null_ptr
      if (present(x0)) xp = c_loc(x0)
      call pfg_check(pfg_solve(this%handle, o, xp, x, info), "solve")
      if (info%status > 0) print *, "[CAUTION] FEMSolverGPU_%solve >> not converged within itrmax"
   end function

   ! FEMSolver_%zeros() (FEMSolverClass.f90:1310-1322)
   subroutine zerosFEMSolverGPU(this)
      class(FEMSolverGPU_), intent(inout) :: this
      call pfg_check(pfg_zeros(this%handle), "zeros")
   end subroutine

   ! FEMSolver_%keepThisMatrixAs(As) (FEMSolverClass.f90:1544-1604)
   subroutine keepThisMatrixAsFEMSolverGPU(this, As)
      class(FEMSolverGPU_), intent(inout) :: this
      character(*), intent(in) :: As
      call pfg_check(pfg_keep_this_matrix_as(this%handle, trim(As)//c_null_char), "keepThisMatrixAs")
   end subroutine

   ! FEMSolver_%loadMatrix(from) (FEMSolverClass.f90:1203-1222)
   subroutine loadMatrixFEMSolverGPU(this, from)
      class(FEMSolverGPU_), intent(inout) :: this
      character(*), intent(in) :: from
      call pfg_check(pfg_load_matrix(this%handle, trim(from)//c_null_char), "loadMatrix")
   end subroutine

   ! FEMSolver_%fix_eig(IDs) (FEMSolverClass.f90:1607-1628)
   subroutine fix_eigFEMSolverGPU(this, IDs)
      class(FEMSolverGPU_), intent(inout) :: this
      integer(int32), intent(in) :: IDs(:)
      call pfg_check(pfg_fix_eig(this%handle, int(size(IDs), c_int64_t), IDs), "fix_eig")
   end subroutine

   ! FEMSolver_%eig([num_eigen], eigen_value, eigen_vectors) (FEMSolverClass.f90:1384-1541):
   ! the dense branch (every pair) unless use_LOBPCG, as the reference
   subroutine eigFEMSolverGPU(this, num_eigen, eigen_value, eigen_vectors)
      class(FEMSolverGPU_), intent(inout) :: this
      integer(int32), optional, intent(in) :: num_eigen
      real(real64), allocatable, intent(inout) :: eigen_value(:)
      real(real64), allocatable, intent(inout) :: eigen_vectors(:, :)
      type(pfg_eig_opts) :: o
      type(pfg_info) :: info
      integer(c_int64_t) :: n, nnz, nred
      integer(c_int32_t) :: m
      call pfg_check(pfg_get_crs_size(this%handle, n, nnz), "eig")
      if (this%use_LOBPCG) then
         m = this%LOBPCG_NUM_MODE
         if (present(num_eigen)) m = num_eigen
         call pfg_eig_opts_default(o)
         o%max_itr = this%LOBPCG_MAX_ITR
         o%tol = this%LOBPCG_TOL
         o%debug = merge(1, 0, this%debug)
         if (allocated(eigen_value)) deallocate (eigen_value)
         if (allocated(eigen_vectors)) deallocate (eigen_vectors)
         allocate (eigen_value(m), eigen_vectors(n, m))
         call pfg_check(pfg_eig(this%handle, o, m, eigen_value, eigen_vectors, info), "eig")
      else
         call pfg_check(pfg_eig_reduced_size(this%handle, nred), "eig")
         m = int(nred, c_int32_t)
         if (present(num_eigen)) m = min(num_eigen, m)
         if (allocated(eigen_value)) deallocate (eigen_value)
         if (allocated(eigen_vectors)) deallocate (eigen_vectors)
         allocate (eigen_value(m), eigen_vectors(n, m))
         call pfg_check(pfg_eig_dense(this%handle, m, eigen_value, eigen_vectors, info), "eig")
      end if
   end subroutine

   ! FEMSolver_%getCRS() (FEMSolverClass.f90:2690-2727): the working matrix into
   ! CRS_Index_Row / CRS_Index_Col / CRS_val and the right-hand side into CRS_RHS
   subroutine getCRSFEMSolverGPU(this)
      class(FEMSolverGPU_), intent(inout) :: this
      integer(c_int64_t) :: n, nnz
      call pfg_check(pfg_get_crs_size(this%handle, n, nnz), "getCRS")
      if (allocated(this%CRS_Index_Row)) deallocate (this%CRS_Index_Row)
      if (allocated(this%CRS_Index_Col)) deallocate (this%CRS_Index_Col)
      if (allocated(this%CRS_val)) deallocate (this%CRS_val)
      if (allocated(this%CRS_RHS)) deallocate (this%CRS_RHS)
      allocate (this%CRS_Index_Row(n + 1), this%CRS_Index_Col(nnz), this%CRS_val(nnz), this%CRS_RHS(n))
      call pfg_check(pfg_get_crs(this%handle, this%CRS_Index_Row, this%CRS_Index_Col, this%CRS_val), "getCRS")
      call pfg_check(pfg_get_rhs(this%handle, n, this%CRS_RHS), "getCRS")
   end subroutine

   ! FEMSolver_%remove() (FEMSolverClass.f90:1827-1889)
   subroutine removeFEMSolverGPU(this)
      class(FEMSolverGPU_), intent(inout) :: this
      if (c_associated(this%handle)) call pfg_check(pfg_destroy(this%handle), "remove")
      this%handle = c_null_ptr
      if (allocated(this%CRS_Index_Row)) deallocate (this%CRS_Index_Row)
      if (allocated(this%CRS_Index_Col)) deallocate (this%CRS_Index_Col)
      if (allocated(this%CRS_val)) deallocate (this%CRS_val)
      if (allocated(this%CRS_RHS)) deallocate (this%CRS_RHS)
   end subroutine

end module FEMSolverGPUClass
