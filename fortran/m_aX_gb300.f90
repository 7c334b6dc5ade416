!> GPU drop-in for the FAS multigrid entry points of m_a$D_mg
!> (src/m_aX_mg.f90:164-255): mg$D_fas_vcycle and mg$D_fas_fmg with the
!> reference's arguments, run by the afivo_gb300 library on the device.
!>
!> The tree stays the caller's a$D_t. On each call this module
!>  * mirrors the tree's topology into a device forest when the refinement
!>    changed since the last call (same base boxes, then refinement replayed
!>    pass by pass until the mirror has the caller's boxes);
!>  * samples mg%sides_bc once per physical-boundary face on a copy of the box
!>    and uploads the type and values (afv_forest_set_bc_faces);
!>  * uploads phi, rhs and tmp of every box, runs the cycle, and downloads
!>    phi, rhs and tmp, so the tree ends as the reference's routine leaves it.
!>
!> Lean mode (gb$D_lean = .true.): the device keeps phi, rhs and tmp between
!> calls. A call uploads (and samples sides_bc) only when the refinement
!> changed or the caller bumped gb$D_data_gen since the last upload (after
!> changing phi, rhs, tmp, eps, the level set, the boundary or operator hooks
!> on the host), and downloads
!> phi only, plus tmp when set_residual is true. The host's rhs and tmp are
!> then out of date where the cycle changed them (the coarse levels' rhs,
!> tmp without set_residual); gb$D_sync downloads all three.
!>
!> The operator hooks may be any of the reference's built-in sets: the
!> Laplacian (the defaults of mg$D_init_mg), mg$D_box_*_lpld,
!> mg2_box_*_clpl(d), mg$D_box_*_lpllsf, or mg$D_auto_* (with
!> mg$D_auto_rstr, or mg$D_box_rstr_lpl when there is no level set), with
!> mg%i_eps, mg%i_lsf and mg%i_bval uploaded beside phi; cylindrical trees
!> (coord_t = a5_cyl) are mirrored as such. Other hooks, and a sides_rb other
!> than mg$D_sides_rb, stop the call.
!>
!> This file is a template like the reference's m_aX_*.f90: the Makefile
!> beside it expands $D to 2 and 3 (sed, then cpp).
module m_a$D_gb300
  use iso_c_binding
  use m_afivo_gb300
  use m_a$D_t
  use m_a$D_mg, only: mg$D_t, mg$D_box_lpl, mg$D_box_gsrb_lpl, &
       mg$D_box_corr_lpl, mg$D_box_rstr_lpl, mg$D_sides_rb, &
       mg$D_box_lpld, mg$D_box_gsrb_lpld, mg$D_box_corr_lpld, &
       mg$D_box_lpllsf, mg$D_box_gsrb_lpllsf, mg$D_box_corr_lpllsf, mg$D_box_rstr_lpllsf, &
#if $D == 2
       mg$D_box_clpl, mg$D_box_gsrb_clpl, mg$D_box_clpld, mg$D_box_gsrb_clpld, &
#endif
       mg$D_auto_op, mg$D_auto_gsrb, mg$D_auto_corr, mg$D_auto_rstr
  implicit none
  private

  !> Device mirror of the last tree used
  type gb_mirror_t
     type(c_ptr)          :: tree = c_null_ptr
     type(c_ptr)          :: forest = c_null_ptr
     integer(c_long_long) :: stamp(4) = -1
     !> gb$D_data_gen at the last upload (-1: none)
     integer(c_long_long) :: gen = -1
     !> reference ids of the mirror's boxes in the host exchange order
     integer, allocatable :: order(:)
     !> extra cell variables added to the forest (eps, lsf, bval)
     logical              :: has_extra = .false.
  end type gb_mirror_t

  type(gb_mirror_t), save      :: mirror
  type(a$D_t), pointer, save   :: cb_tree => null()

  !> CUDA device the mirror is created on
  integer, public :: gb$D_device = 0
  !> Keep the state on the device between calls (see above)
  logical, public :: gb$D_lean = .false.
  !> Bumped by the caller whenever it changes phi, rhs, tmp, sides_bc, the
  !> operator hooks or their variables (eps, lsf, bval)
  integer(c_long_long), public :: gb$D_data_gen = 0

  public :: mg$D_fas_vcycle
  public :: mg$D_fas_fmg
  public :: gb$D_release
  public :: gb$D_sync

contains

  !> mg$D_fas_vcycle (src/m_aX_mg.f90:208-255) on the device
  subroutine mg$D_fas_vcycle(tree, mg, highest_lvl, set_residual)
    type(a$D_t), intent(inout), target :: tree
    type(mg$D_t), intent(in)           :: mg
    integer, intent(in)                :: highest_lvl
    logical, intent(in)                :: set_residual
    type(afv_mg_opts)                  :: opts

    call prepare(tree, mg, opts)
    call afv_check(afv_mg_fas_vcycle(mirror%forest, opts, int(highest_lvl, c_int), &
         merge(1_c_int, 0_c_int, set_residual)), "mg$D_fas_vcycle")
    call download_after(tree, mg, set_residual)
  end subroutine mg$D_fas_vcycle

  !> mg$D_fas_fmg (src/m_aX_mg.f90:164-203) on the device
  subroutine mg$D_fas_fmg(tree, mg, set_residual, have_guess)
    type(a$D_t), intent(inout), target :: tree
    type(mg$D_t), intent(in)           :: mg
    logical, intent(in)                :: set_residual
    logical, intent(in)                :: have_guess
    type(afv_mg_opts)                  :: opts

    call prepare(tree, mg, opts)
    call afv_check(afv_mg_fas_fmg(mirror%forest, opts, merge(1_c_int, 0_c_int, set_residual), &
         merge(1_c_int, 0_c_int, have_guess)), "mg$D_fas_fmg")
    call download_after(tree, mg, set_residual)
  end subroutine mg$D_fas_fmg

  !> Download phi, rhs and tmp of the mirror into the tree (after lean calls)
  subroutine gb$D_sync(tree, mg)
    type(a$D_t), intent(inout) :: tree
    type(mg$D_t), intent(in)   :: mg
    if (.not. c_associated(mirror%forest)) return
    call download_all(tree, mg)
  end subroutine gb$D_sync

  !> Free the device mirror (the next call builds it again)
  subroutine gb$D_release()
    if (c_associated(mirror%forest)) call afv_forest_destroy(mirror%forest)
    if (c_associated(mirror%tree)) call afv_tree_destroy(mirror%tree)
    mirror%forest = c_null_ptr
    mirror%tree = c_null_ptr
    mirror%stamp = -1
    mirror%gen = -1
    mirror%has_extra = .false.
    if (allocated(mirror%order)) deallocate(mirror%order)
  end subroutine gb$D_release

  subroutine prepare(tree, mg, opts)
    type(a$D_t), intent(inout), target :: tree
    type(mg$D_t), intent(in)           :: mg
    type(afv_mg_opts), intent(out)     :: opts
    integer(c_long_long)               :: stamp(4)

    integer(c_int)                     :: op

    if (.not. mg%initialized) stop "afivo_gb300: call mg$D_init_mg first"
    if (.not. associated(mg%sides_rb, mg$D_sides_rb)) &
         stop "afivo_gb300: only mg$D_sides_rb runs on the device"
    op = operator_of(mg)

    call tree_stamp(tree, stamp)
    if (any(stamp /= mirror%stamp)) then
       call build_mirror(tree)
       mirror%stamp = stamp
    end if
    if (.not. gb$D_lean .or. mirror%gen /= gb$D_data_gen) then
       call sample_bc(tree, mg)
       call upload(tree, mg%i_phi, AFV_PHI)
       call upload(tree, mg%i_rhs, AFV_RHS)
       call upload(tree, mg%i_tmp, AFV_TMP)
       if (op /= AFV_OP_LPL .and. .not. mirror%has_extra) then
          call afv_check(afv_forest_add_vars(mirror%forest, 3_c_int, 0_c_int), "afv_forest_add_vars")
          mirror%has_extra = .true.
       end if
       ! eps, lsf and bval as the forest's cell variables 3, 4 and 5; the
       ! auto tags are taken from them by afv_mg_set_operator_lsf
       if (mg%i_eps > 0 .and. op /= AFV_OP_LPL) call upload(tree, mg%i_eps, 3_c_int)
       if (mg%i_lsf > 0 .and. op /= AFV_OP_LPL) then
          call upload(tree, mg%i_lsf, 4_c_int)
          call upload(tree, mg%i_bval, 5_c_int)
       end if
       call afv_check(afv_mg_set_operator_lsf(mirror%forest, op, &
            merge(3_c_int, -1_c_int, mg%i_eps > 0 .and. op /= AFV_OP_LPL), &
            merge(4_c_int, -1_c_int, mg%i_lsf > 0 .and. op /= AFV_OP_LPL), &
            merge(5_c_int, -1_c_int, mg%i_lsf > 0 .and. op /= AFV_OP_LPL)), "afv_mg_set_operator_lsf")
       mirror%gen = gb$D_data_gen
    end if
    opts%n_cycle_down = mg%n_cycle_down
    opts%n_cycle_up = mg%n_cycle_up
    opts%n_cycle_base = mg%n_cycle_base
  end subroutine prepare

  !> The library's operator for the caller's hooks (mg%box_op, box_gsrb,
  !> box_corr, box_rstr), or a stop when the set is not a built-in one
  integer(c_int) function operator_of(mg) result(op)
    type(mg$D_t), intent(in) :: mg
    logical                  :: rstr_lpl
    rstr_lpl = associated(mg%box_rstr, mg$D_box_rstr_lpl)
    op = -1
    if (associated(mg%box_op, mg$D_box_lpl) .and. associated(mg%box_gsrb, mg$D_box_gsrb_lpl) .and. &
         associated(mg%box_corr, mg$D_box_corr_lpl) .and. rstr_lpl) then
       op = AFV_OP_LPL
    else if (associated(mg%box_op, mg$D_box_lpld) .and. associated(mg%box_gsrb, mg$D_box_gsrb_lpld) .and. &
         associated(mg%box_corr, mg$D_box_corr_lpld) .and. rstr_lpl) then
       op = AFV_OP_LPLD
    else if (associated(mg%box_op, mg$D_box_lpllsf) .and. associated(mg%box_gsrb, mg$D_box_gsrb_lpllsf) .and. &
         associated(mg%box_corr, mg$D_box_corr_lpllsf) .and. associated(mg%box_rstr, mg$D_box_rstr_lpllsf)) then
       op = AFV_OP_LPLLSF
    else if (associated(mg%box_op, mg$D_auto_op) .and. associated(mg%box_gsrb, mg$D_auto_gsrb) .and. &
         associated(mg%box_corr, mg$D_auto_corr) .and. (associated(mg%box_rstr, mg$D_auto_rstr) .or. &
         (rstr_lpl .and. mg%i_lsf < 0))) then
       op = AFV_OP_AUTO
#if $D == 2
    else if (associated(mg%box_op, mg$D_box_clpl) .and. associated(mg%box_gsrb, mg$D_box_gsrb_clpl) .and. &
         associated(mg%box_corr, mg$D_box_corr_lpl) .and. rstr_lpl) then
       op = AFV_OP_CLPL
    else if (associated(mg%box_op, mg$D_box_clpld) .and. associated(mg%box_gsrb, mg$D_box_gsrb_clpld) .and. &
         associated(mg%box_corr, mg$D_box_corr_lpld) .and. rstr_lpl) then
       op = AFV_OP_CLPLD
#endif
    end if
    if (op < 0) stop "afivo_gb300: these operator hooks do not run on the device"
  end function operator_of

  !> What a call hands back: everything, or in lean mode phi (and tmp when
  !> the residual was asked for)
  subroutine download_after(tree, mg, set_residual)
    type(a$D_t), intent(inout) :: tree
    type(mg$D_t), intent(in)   :: mg
    logical, intent(in)        :: set_residual
    if (.not. gb$D_lean) then
       call download_all(tree, mg)
    else
       call download(tree, mg%i_phi, AFV_PHI)
       if (set_residual) call download(tree, mg%i_tmp, AFV_TMP)
    end if
  end subroutine download_after

  subroutine download_all(tree, mg)
    type(a$D_t), intent(inout) :: tree
    type(mg$D_t), intent(in)   :: mg
    call download(tree, mg%i_phi, AFV_PHI)
    call download(tree, mg%i_rhs, AFV_RHS)
    call download(tree, mg%i_tmp, AFV_TMP)
  end subroutine download_all

  !> A fingerprint of the tree's refinement
  subroutine tree_stamp(tree, stamp)
    type(a$D_t), intent(in)           :: tree
    integer(c_long_long), intent(out) :: stamp(4)
    integer                           :: id
    stamp(1) = tree%highest_id
    stamp(2) = tree%highest_lvl
    stamp(3:4) = 0
    do id = 1, tree%highest_id
       if (.not. tree%boxes(id)%in_use) cycle
       stamp(3) = stamp(3) + 1
       if (tree%boxes(id)%children(1) /= a5_no_box) &
            stamp(4) = stamp(4) + int(id, c_long_long) * (tree%boxes(id)%lvl + 7)
    end do
  end subroutine tree_stamp

  !> floor((i - 1) / 2**k) + 1: the index of the ancestor k levels up
  elemental integer function ancestor_ix(i, k)
    integer, intent(in) :: i, k
    ancestor_ix = (i - 1 - modulo(i - 1, 2**k)) / 2**k + 1
  end function ancestor_ix

  !> Id of the caller's box at (lvl, ix), or 0 if it does not exist
  integer function find_box(tree, lvl, ix) result(id)
    type(a$D_t), intent(in) :: tree
    integer, intent(in)     :: lvl, ix($D)
    integer                 :: n, l, i, top

    id = 0
    top = min(lvl, 1)
    do n = 1, size(tree%lvls(top)%ids)
       i = tree%lvls(top)%ids(n)
       if (all(tree%boxes(i)%ix == ancestor_ix(ix, lvl - top))) then
          id = i
          exit
       end if
    end do
    do l = 2, lvl
       if (id == 0) return
       if (tree%boxes(id)%children(1) == a5_no_box) then
          id = 0
          return
       end if
       id = tree%boxes(id)%children(a$D_ix_to_ichild(ancestor_ix(ix, lvl - l)))
    end do
  end function find_box

  !> Refinement callback of the replay: refine where the caller's tree has
  !> children
  subroutine replay_flag(box, ref_flag, user) bind(C)
    type(afv_box_view), intent(in) :: box
    integer(c_int), intent(out)    :: ref_flag
    type(c_ptr), value             :: user
    integer                        :: id

    ref_flag = AFV_KEEP_REF
    if (box%lvl < 1) return
    id = find_box(cb_tree, int(box%lvl), int(box%ix(1:$D)))
    if (id > 0) then
       if (cb_tree%boxes(id)%children(1) /= a5_no_box) ref_flag = AFV_DO_REF
    end if
  end subroutine replay_flag

  subroutine build_mirror(tree)
    type(a$D_t), intent(inout), target :: tree
    integer                            :: min_lvl, coarsen_to, n_base, n, nb, k, lvl, m
    integer(c_int)                     :: n_add, n_rm, info(8), sizes(3)
    integer(c_int), allocatable        :: ix_list(:, :), nb_list(:, :), pos(:)
    integer(c_int), allocatable, target :: ids(:)
    integer(c_int), allocatable        :: e_lvl(:), e_ix(:, :), e_parent(:), e_children(:, :)
    integer(c_int), allocatable        :: e_nb(:, :), e_nc(:), e_use(:)
    real(c_double), allocatable        :: e_dr(:), e_rmin(:, :)
    type(c_ptr)                        :: trees(1)
    type(afv_forest_opts)              :: fo

    call gb$D_release()
    min_lvl = lbound(tree%lvls, 1)
    coarsen_to = -1
    if (min_lvl < 1) coarsen_to = tree%n_cell / 2**(1 - min_lvl)
    call afv_check(afv_tree_create($D, int(tree%n_cell, c_int), real(tree%dr_base, c_double), &
         real(tree%r_base, c_double), int(tree%lvl_limit, c_int), int(coarsen_to, c_int), &
         1024.0_c_double, mirror%tree), "afv_tree_create")
    if (tree%coord_t == a5_cyl) &
         call afv_check(afv_tree_set_coord(mirror%tree, AFV_COORD_CYL), "afv_tree_set_coord")

    ! Base boxes in the order of the caller's level-1 list; neighbours as
    ! positions in that list, physical boundaries unchanged.
    n_base = size(tree%lvls(1)%ids)
    allocate(ix_list($D, n_base), nb_list(a$D_num_neighbors, n_base), pos(tree%highest_id))
    pos = 0
    do n = 1, n_base
       pos(tree%lvls(1)%ids(n)) = n
    end do
    do n = 1, n_base
       ix_list(:, n) = tree%boxes(tree%lvls(1)%ids(n))%ix
       do nb = 1, a$D_num_neighbors
          k = tree%boxes(tree%lvls(1)%ids(n))%neighbors(nb)
          if (k > a5_no_box) then
             nb_list(nb, n) = pos(k)
          else
             nb_list(nb, n) = k
          end if
       end do
    end do
    call afv_check(afv_tree_set_base(mirror%tree, int(n_base, c_int), ix_list, nb_list), &
         "afv_tree_set_base")

    cb_tree => tree
    do
       call afv_check(afv_tree_adjust_refinement(mirror%tree, c_funloc(replay_flag), &
            c_null_ptr, n_add, n_rm), "afv_tree_adjust_refinement")
       if (n_add == 0) exit
    end do
    nullify(cb_tree)

    ! Host exchange order of the mirror, as ids of the caller's tree
    call afv_check(afv_tree_get_info(mirror%tree, info), "afv_tree_get_info")
    allocate(e_lvl(info(5)), e_ix($D, info(5)), e_parent(info(5)), &
         e_children(2**$D, info(5)), e_nb(2*$D, info(5)), e_nc(info(5)), e_use(info(5)), &
         e_dr(info(5)), e_rmin($D, info(5)))
    call afv_check(afv_tree_export(mirror%tree, e_lvl, e_ix, e_parent, e_children, e_nb, &
         e_nc, e_dr, e_rmin, e_use), "afv_tree_export")
    allocate(mirror%order(info(6)))
    m = 0
    do lvl = info(3), info(4)
       call afv_check(afv_tree_level(mirror%tree, int(lvl, c_int), sizes, c_null_ptr, &
            c_null_ptr, c_null_ptr), "afv_tree_level")
       if (sizes(1) == 0) cycle
       allocate(ids(sizes(1)))
       call afv_check(afv_tree_level(mirror%tree, int(lvl, c_int), sizes, c_loc(ids), &
            c_null_ptr, c_null_ptr), "afv_tree_level")
       do n = 1, sizes(1)
          m = m + 1
          mirror%order(m) = find_box(tree, lvl, int(e_ix(1:$D, ids(n))))
          if (mirror%order(m) == 0) stop "afivo_gb300: mirror differs from the tree"
       end do
       deallocate(ids)
    end do
    if (m /= size(mirror%order)) stop "afivo_gb300: mirror box count differs"

    trees(1) = mirror%tree
    fo%device = gb$D_device
    fo%mixed_buffers = 0
    call afv_check(afv_forest_create(1_c_int, trees, fo, mirror%forest), "afv_forest_create")
  end subroutine build_mirror

  !> Number of values of the boxes of the mirror order
  integer(c_long_long) function n_values(tree) result(n)
    type(a$D_t), intent(in) :: tree
    integer                 :: m
    n = 0
    do m = 1, size(mirror%order)
       n = n + int(tree%boxes(mirror%order(m))%n_cell + 2, c_long_long)**$D
    end do
  end function n_values

  subroutine upload(tree, iv, var)
    type(a$D_t), intent(in)     :: tree
    integer, intent(in)         :: iv
    integer(c_int), intent(in)  :: var
    real(c_double), allocatable :: buf(:)
    integer(c_long_long)        :: k
    integer                     :: m, id, nv

    allocate(buf(n_values(tree)))
    k = 0
    do m = 1, size(mirror%order)
       id = mirror%order(m)
       nv = (tree%boxes(id)%n_cell + 2)**$D
#if $D == 2
       buf(k+1:k+nv) = reshape(tree%boxes(id)%cc(:, :, iv), [nv])
#elif $D == 3
       buf(k+1:k+nv) = reshape(tree%boxes(id)%cc(:, :, :, iv), [nv])
#endif
       k = k + nv
    end do
    call afv_check(afv_forest_set_var(mirror%forest, 0_c_int, var, buf, 0_c_int), &
         "afv_forest_set_var")
  end subroutine upload

  subroutine download(tree, iv, var)
    type(a$D_t), intent(inout)  :: tree
    integer, intent(in)         :: iv
    integer(c_int), intent(in)  :: var
    real(c_double), allocatable :: buf(:)
    integer(c_long_long)        :: k
    integer                     :: m, id, ng

    allocate(buf(n_values(tree)))
    call afv_check(afv_forest_get_var(mirror%forest, 0_c_int, var, buf, 0_c_int), &
         "afv_forest_get_var")
    k = 0
    do m = 1, size(mirror%order)
       id = mirror%order(m)
       ng = tree%boxes(id)%n_cell + 2
#if $D == 2
       tree%boxes(id)%cc(:, :, iv) = reshape(buf(k+1:k+ng**2), [ng, ng])
#elif $D == 3
       tree%boxes(id)%cc(:, :, :, iv) = reshape(buf(k+1:k+ng**3), [ng, ng, ng])
#endif
       k = k + ng**$D
    end do
  end subroutine download

  !> The boundary values a sides_bc hook wrote into the ghost face nb of box
  subroutine face_values(box, nb, iv, v)
    type(box$D_t), intent(in)   :: box
    integer, intent(in)         :: nb, iv
    real(c_double), intent(out) :: v(:)
    integer                     :: nc
    nc = box%n_cell
#if $D == 2
    select case (nb)
    case (1)
       v = box%cc(0, 1:nc, iv)
    case (2)
       v = box%cc(nc+1, 1:nc, iv)
    case (3)
       v = box%cc(1:nc, 0, iv)
    case (4)
       v = box%cc(1:nc, nc+1, iv)
    end select
#elif $D == 3
    select case (nb)
    case (1)
       v = reshape(box%cc(0, 1:nc, 1:nc, iv), [nc*nc])
    case (2)
       v = reshape(box%cc(nc+1, 1:nc, 1:nc, iv), [nc*nc])
    case (3)
       v = reshape(box%cc(1:nc, 0, 1:nc, iv), [nc*nc])
    case (4)
       v = reshape(box%cc(1:nc, nc+1, 1:nc, iv), [nc*nc])
    case (5)
       v = reshape(box%cc(1:nc, 1:nc, 0, iv), [nc*nc])
    case (6)
       v = reshape(box%cc(1:nc, 1:nc, nc+1, iv), [nc*nc])
    end select
#endif
  end subroutine face_values

  !> Call mg%sides_bc once per physical-boundary face, on a copy of the box,
  !> and upload the returned types and values
  subroutine sample_bc(tree, mg)
    type(a$D_t), intent(in)     :: tree
    type(mg$D_t), intent(in)    :: mg
    type(box$D_t)               :: scratch
    integer(c_int), allocatable :: types(:)
    real(c_double), allocatable :: vals(:)
    integer(c_long_long)        :: nf, nv
    integer                     :: m, id, nb, nfc, bc_type

    nf = 0
    nv = 0
    do m = 1, size(mirror%order)
       id = mirror%order(m)
       do nb = 1, a$D_num_neighbors
          if (tree%boxes(id)%neighbors(nb) < a5_no_box) then
             nf = nf + 1
             nv = nv + tree%boxes(id)%n_cell**($D-1)
          end if
       end do
    end do
    allocate(types(nf), vals(nv))
    nf = 0
    nv = 0
    do m = 1, size(mirror%order)
       id = mirror%order(m)
       do nb = 1, a$D_num_neighbors
          if (tree%boxes(id)%neighbors(nb) >= a5_no_box) cycle
          scratch = tree%boxes(id)
          call mg%sides_bc(scratch, nb, mg%i_phi, bc_type)
          nfc = scratch%n_cell**($D-1)
          nf = nf + 1
          types(nf) = int(bc_type, c_int)  ! a5_bc_dirichlet / a5_bc_neumann = AFV_BC_*
          call face_values(scratch, nb, mg%i_phi, vals(nv+1:nv+nfc))
          nv = nv + nfc
       end do
    end do
    call afv_check(afv_forest_set_bc_faces(mirror%forest, 0_c_int, nf, types, nv, vals), &
         "afv_forest_set_bc_faces")
  end subroutine sample_bc

end module m_a$D_gb300
