!> iso_c_binding interfaces of the afivo_gb300 C library
!> (include/afivo_gb300.h). Dimension-independent; the drop-in routines with
!> the reference's names are in m_aX_gb300.f90 (expanded to m_a2_gb300 and
!> m_a3_gb300 by the Makefile beside this file).
module m_afivo_gb300
  use iso_c_binding
  implicit none
  public

  integer(c_int), parameter :: AFV_OK = 0
  integer(c_int), parameter :: AFV_ERR_INVALID = -1
  integer(c_int), parameter :: AFV_ERR_CUDA = -2
  integer(c_int), parameter :: AFV_ERR_NOMEM = -3
  integer(c_int), parameter :: AFV_ERR_UNSUPPORTED = -4
  integer(c_int), parameter :: AFV_ERR_TIMEOUT = -5
  integer(c_int), parameter :: AFV_ERR_STATE = -6
  integer(c_int), parameter :: AFV_ERR_BUDGET = -7
  integer(c_int), parameter :: AFV_ERR_DIVERGED = -8
  integer(c_int), parameter :: AFV_ERR_NOT_CONVERGED = -9

  integer(c_int), parameter :: AFV_RM_REF = -1, AFV_KEEP_REF = 0, AFV_DO_REF = 1
  integer(c_int), parameter :: AFV_PHI = 0, AFV_RHS = 1, AFV_TMP = 2
  integer(c_int), parameter :: AFV_BC_DIRICHLET = -1, AFV_BC_NEUMANN = -2
  integer(c_int), parameter :: AFV_PREC_FP64 = 0, AFV_PREC_MIXED = 1
  integer(c_int), parameter :: AFV_OP_LPL = 0, AFV_OP_LPLD = 1, AFV_OP_AUTO = 2
  integer(c_int), parameter :: AFV_OP_CLPL = 3, AFV_OP_CLPLD = 4, AFV_OP_LPLLSF = 5
  integer(c_int), parameter :: AFV_COORD_XYZ = 0, AFV_COORD_CYL = 1

  !> What a refinement callback sees of a box (afv_box_view)
  type, bind(C) :: afv_box_view
     integer(c_int) :: id, lvl, n_cell, dim
     integer(c_int) :: ix(3)
     real(c_double) :: dr
     real(c_double) :: r_min(3)
     integer(c_int) :: pass
  end type afv_box_view

  !> Multigrid options (afv_mg_opts); negative counts mean the defaults (2)
  type, bind(C) :: afv_mg_opts
     integer(c_int) :: n_cycle_down = -1
     integer(c_int) :: n_cycle_up = -1
     integer(c_int) :: n_cycle_base = -1
  end type afv_mg_opts

  type, bind(C) :: afv_forest_opts
     integer(c_int) :: device = 0
     integer(c_int) :: mixed_buffers = 0
  end type afv_forest_opts

  interface
     function afv_last_error() bind(C, name="afv_last_error") result(msg)
       import :: c_ptr
       type(c_ptr) :: msg
     end function afv_last_error

     function afv_tree_create(dim, n_cell, dr, r_min, lvl_limit, coarsen_to, &
          mem_limit_gb, tree) bind(C, name="afv_tree_create") result(rc)
       import :: c_int, c_double, c_ptr
       integer(c_int), value      :: dim, n_cell, lvl_limit, coarsen_to
       real(c_double), value      :: dr, mem_limit_gb
       real(c_double), intent(in) :: r_min(*)
       type(c_ptr), intent(out)   :: tree
       integer(c_int)             :: rc
     end function afv_tree_create

     function afv_tree_set_coord(tree, coord) bind(C, name="afv_tree_set_coord") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value    :: tree
       integer(c_int), value :: coord
       integer(c_int)        :: rc
     end function afv_tree_set_coord

     function afv_tree_set_base(tree, n_boxes, ix_list, nb_list) &
          bind(C, name="afv_tree_set_base") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value         :: tree
       integer(c_int), value      :: n_boxes
       integer(c_int), intent(in) :: ix_list(*), nb_list(*)
       integer(c_int)             :: rc
     end function afv_tree_set_base

     function afv_tree_adjust_refinement(tree, fn, user, n_add, n_rm) &
          bind(C, name="afv_tree_adjust_refinement") result(rc)
       import :: c_int, c_ptr, c_funptr
       type(c_ptr), value          :: tree
       type(c_funptr), value       :: fn
       type(c_ptr), value          :: user
       integer(c_int), intent(out) :: n_add, n_rm
       integer(c_int)              :: rc
     end function afv_tree_adjust_refinement

     subroutine afv_tree_destroy(tree) bind(C, name="afv_tree_destroy")
       import :: c_ptr
       type(c_ptr), value :: tree
     end subroutine afv_tree_destroy

     function afv_tree_get_info(tree, out8) bind(C, name="afv_tree_get_info") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value          :: tree
       integer(c_int), intent(out) :: out8(8)
       integer(c_int)              :: rc
     end function afv_tree_get_info

     function afv_tree_export(tree, lvl, ix, parent, children, neighbors, n_cell, dr, &
          r_min, in_use) bind(C, name="afv_tree_export") result(rc)
       import :: c_int, c_double, c_ptr
       type(c_ptr), value          :: tree
       integer(c_int), intent(out) :: lvl(*), ix(*), parent(*), children(*), neighbors(*)
       integer(c_int), intent(out) :: n_cell(*), in_use(*)
       real(c_double), intent(out) :: dr(*), r_min(*)
       integer(c_int)              :: rc
     end function afv_tree_export

     function afv_tree_level(tree, lvl, sizes3, ids, leaves, parents) &
          bind(C, name="afv_tree_level") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value          :: tree
       integer(c_int), value       :: lvl
       integer(c_int), intent(out) :: sizes3(3)
       type(c_ptr), value          :: ids, leaves, parents
       integer(c_int)              :: rc
     end function afv_tree_level

     function afv_forest_create(n_trees, trees, opts, forest) &
          bind(C, name="afv_forest_create") result(rc)
       import :: c_int, c_ptr, afv_forest_opts
       integer(c_int), value               :: n_trees
       type(c_ptr), intent(in)             :: trees(*)
       type(afv_forest_opts), intent(in)   :: opts
       type(c_ptr), intent(out)            :: forest
       integer(c_int)                      :: rc
     end function afv_forest_create

     subroutine afv_forest_destroy(forest) bind(C, name="afv_forest_destroy")
       import :: c_ptr
       type(c_ptr), value :: forest
     end subroutine afv_forest_destroy

     function afv_forest_add_vars(forest, n_cc, n_fc) bind(C, name="afv_forest_add_vars") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value    :: forest
       integer(c_int), value :: n_cc, n_fc
       integer(c_int)        :: rc
     end function afv_forest_add_vars

     function afv_mg_set_operator_lsf(forest, op, i_eps, i_lsf, i_bval) &
          bind(C, name="afv_mg_set_operator_lsf") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value    :: forest
       integer(c_int), value :: op, i_eps, i_lsf, i_bval
       integer(c_int)        :: rc
     end function afv_mg_set_operator_lsf

     function afv_forest_set_var(forest, tree, var, host, interior_only) &
          bind(C, name="afv_forest_set_var") result(rc)
       import :: c_int, c_double, c_ptr
       type(c_ptr), value         :: forest
       integer(c_int), value      :: tree, var, interior_only
       real(c_double), intent(in) :: host(*)
       integer(c_int)             :: rc
     end function afv_forest_set_var

     function afv_forest_get_var(forest, tree, var, host, interior_only) &
          bind(C, name="afv_forest_get_var") result(rc)
       import :: c_int, c_double, c_ptr
       type(c_ptr), value          :: forest
       integer(c_int), value       :: tree, var, interior_only
       real(c_double), intent(out) :: host(*)
       integer(c_int)              :: rc
     end function afv_forest_get_var

     function afv_forest_set_bc_faces(forest, tree, n_faces, bc_type, n_values, values) &
          bind(C, name="afv_forest_set_bc_faces") result(rc)
       import :: c_int, c_long_long, c_double, c_ptr
       type(c_ptr), value          :: forest
       integer(c_int), value       :: tree
       integer(c_long_long), value :: n_faces, n_values
       integer(c_int), intent(in)  :: bc_type(*)
       real(c_double), intent(in)  :: values(*)
       integer(c_int)              :: rc
     end function afv_forest_set_bc_faces

     function afv_mg_init(mg) bind(C, name="afv_mg_init") result(rc)
       import :: c_int, afv_mg_opts
       type(afv_mg_opts), intent(inout) :: mg
       integer(c_int)                   :: rc
     end function afv_mg_init

     function afv_mg_fas_vcycle(forest, mg, highest_lvl, set_residual) &
          bind(C, name="afv_mg_fas_vcycle") result(rc)
       import :: c_int, c_ptr, afv_mg_opts
       type(c_ptr), value            :: forest
       type(afv_mg_opts), intent(in) :: mg
       integer(c_int), value         :: highest_lvl, set_residual
       integer(c_int)                :: rc
     end function afv_mg_fas_vcycle

     function afv_mg_fas_fmg(forest, mg, set_residual, have_guess) &
          bind(C, name="afv_mg_fas_fmg") result(rc)
       import :: c_int, c_ptr, afv_mg_opts
       type(c_ptr), value            :: forest
       type(afv_mg_opts), intent(in) :: mg
       integer(c_int), value         :: set_residual, have_guess
       integer(c_int)                :: rc
     end function afv_mg_fas_fmg

     function afv_mg_solve(forest, mg, precision, tol, max_cycles, cycles, rel_res) &
          bind(C, name="afv_mg_solve") result(rc)
       import :: c_int, c_double, c_ptr, afv_mg_opts
       type(c_ptr), value            :: forest
       type(afv_mg_opts), intent(in) :: mg
       integer(c_int), value         :: precision, max_cycles
       real(c_double), value         :: tol
       integer(c_int), intent(out)   :: cycles(*)
       real(c_double), intent(out)   :: rel_res(*)
       integer(c_int)                :: rc
     end function afv_mg_solve

     function afv_tree_max_abs_cc(forest, tree, var, out) &
          bind(C, name="afv_tree_max_abs_cc") result(rc)
       import :: c_int, c_double, c_ptr
       type(c_ptr), value          :: forest
       integer(c_int), value       :: tree, var
       real(c_double), intent(out) :: out
       integer(c_int)              :: rc
     end function afv_tree_max_abs_cc

     function c_strlen(s) bind(C, name="strlen") result(n)
       import :: c_ptr, c_size_t
       type(c_ptr), value :: s
       integer(c_size_t)  :: n
     end function c_strlen
  end interface

contains

  !> The message of the calling thread's last failure
  function afv_error_message() result(msg)
    character(len=:), allocatable :: msg
    type(c_ptr)                   :: p
    character(kind=c_char), pointer :: chars(:)
    integer                       :: n, i
    p = afv_last_error()
    n = int(c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: msg)
    do i = 1, n
       msg(i:i) = chars(i)
    end do
  end function afv_error_message

  !> Stop with the library's message when rc is not AFV_OK (the reference
  !> stops on errors; callers that want the code call the C functions)
  subroutine afv_check(rc, where)
    integer(c_int), intent(in)   :: rc
    character(len=*), intent(in) :: where
    if (rc /= AFV_OK) then
       print *, where, ": afivo_gb300 error ", rc, ": ", afv_error_message()
       error stop "afivo_gb300 call failed"
    end if
  end subroutine afv_check

end module m_afivo_gb300
