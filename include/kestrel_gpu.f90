! kestrel_gpu.f90 -- the Fortran binding of include/kestrel_gpu.h (ISO_C_BINDING), the
! module a Kestrel host adds to call the GB300 hot path, in the style of the reference's
! own C bindings (src/GeoTiffRead.f90:43-100 with src/RasterData.h, src/version.f90:25-33
! with src/cversion.cpp:28-34).  Derived types mirror the C structs field for field;
! scalars pass by value, arrays and structs by reference, the context as type(c_ptr).
! kg_check maps a nonzero status to the reference's FatalErrorMessage (src/Messages.f90).
module kestrel_gpu
   use, intrinsic :: iso_c_binding
   implicit none
   ! Field for field the structs of include/kestrel_gpu.h (generated from the ctypes mirror
   ! in kestrel_gb300/abi.py, whose sizes and offsets tests/test_abi.py checks against the
   ! C header).  Leading underscores of the C padding fields are dropped: Fortran names
   ! cannot start with one.  The array bounds are KG_MAX_SERIES, KG_MAX_CAPS,
   ! KG_MAX_CUBES, KG_MAX_SOURCES and KG_MAX_TOPO_PARAMS.
   type, bind(C) :: kg_cap
      real(c_double) :: x, y, radius, height, psi, u, v
      integer(c_int32_t) :: shape, pad
   end type
   type, bind(C) :: kg_cube
      real(c_double) :: x, y, length, width, height, psi, u, v
      integer(c_int32_t) :: shape, pad
   end type
   type, bind(C) :: kg_flux_source
      real(c_double) :: x, y, radius
      integer(c_int32_t) :: n_series, pad
      real(c_double) :: time(64), flux(64), psi(64)
   end type
   type, bind(C) :: kg_params
      integer(c_int32_t) :: nXtiles, nYtiles, nXpertile, nYpertile
      real(c_double) :: Xtilesize, Ytilesize
      integer(c_int32_t) :: bcs, pad0
      real(c_double) :: bcsHnval, bcsuval, bcsvval, bcspsival
      integer(c_int32_t) :: geometric_factors, MorphodynamicsOn
      real(c_double) :: g, rhow, rhos, ChezyCo, ManningCo, CoulombCo, PouliquenMinSlope
      real(c_double) :: PouliquenMaxSlope, PouliquenIntermediateSlope, PouliquenBeta
      real(c_double) :: Edwards2019betastar, Edwards2019kappa, Edwards2019Gamma
      real(c_double) :: VoellmySwitchRate, VoellmySwitchValue, EroRate, EroRateGranular
      real(c_double) :: EroDepth, EroCriticalHeight, BedPorosity, maxPack, SolidDiameter
      real(c_double) :: EddyViscosity
      integer(c_int32_t) :: ws0_given, pad1
      real(c_double) :: ws0
      integer(c_int32_t) :: drag, erosion, deposition, erosion_transition, morpho_damping
      integer(c_int32_t) :: fswitch, limiter, TileBuffer
      real(c_double) :: heightThreshold, cfl, maxdt, tstart, tend, SpongeStrength
      integer(c_int32_t) :: Nout, pad2, nCaps, nCubes, nSources, pad3
      type(kg_cap) :: caps(16)
      type(kg_cube) :: cubes(16)
      type(kg_flux_source) :: sources(16)
      integer(c_int32_t) :: topog, n_topog_params
      real(c_double) :: topog_params(8)
   end type
   type, bind(C) :: kg_raster           ! filled from FortranRasterData (src/RasterData.h)
      integer(c_int64_t) :: nx, ny       ! RasterXSize, RasterYSize
      real(c_double) :: origin_x, origin_y, pixel_w, pixel_h, nodata
      real(c_double) :: center_e, center_n   ! RunParams%centerUTM
   end type
   type, bind(C) :: kg_step_stats
      real(c_double) :: t, dt
      integer(c_int64_t) :: steps, rejected, cell_updates
      integer(c_int32_t) :: n_active, n_ghost
      integer(c_int64_t) :: kernel_launches
   end type
   interface
      integer(c_int) function kg_create(params, precision, ctx) bind(C, name="kg_create")
         import :: c_int, c_int32_t, c_ptr
         type(c_ptr), value :: params          ! c_loc(a kg_params variable)
         integer(c_int32_t), value :: precision
         type(c_ptr) :: ctx
      end function
      integer(c_int) function kg_upload_b0(ctx, b0, nx1, ny1) bind(C, name="kg_upload_b0")
         import :: c_int, c_int64_t, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double), intent(in) :: b0(*)
         integer(c_int64_t), value :: nx1, ny1
      end function
      integer(c_int) function kg_upload_raster(ctx, values, geo) bind(C, name="kg_upload_raster")
         import :: c_int, c_ptr, c_double, kg_raster
         type(c_ptr), value :: ctx
         real(c_double), intent(in) :: values(*)   ! RasterIO order: rows from the north, x fastest
         type(kg_raster), intent(in) :: geo
      end function
      integer(c_int) function kg_load_sources(ctx) bind(C, name="kg_load_sources")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
      end function
      integer(c_int) function kg_integrate_to(ctx, tend, stats) bind(C, name="kg_integrate_to")
         import :: c_int, c_ptr, c_double, kg_step_stats
         type(c_ptr), value :: ctx
         real(c_double), value :: tend
         type(kg_step_stats) :: stats
      end function
      integer(c_int) function kg_volume(ctx, out) bind(C, name="kg_volume")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double) :: out(4)
      end function
      integer(c_int) function kg_get_tile_field(ctx, tile, field, out) bind(C, name="kg_get_tile_field")
         import :: c_int, c_int32_t, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: tile, field
         real(c_double) :: out(*)
      end function
      integer(c_int) function kg_step(ctx, t_stop, stats) bind(C, name="kg_step")
         import :: c_int, c_ptr, c_double, kg_step_stats
         type(c_ptr), value :: ctx
         real(c_double), value :: t_stop
         type(kg_step_stats) :: stats
      end function
      integer(c_int) function kg_run(ctx, stats) bind(C, name="kg_run")
         import :: c_int, c_ptr, kg_step_stats
         type(c_ptr), value :: ctx
         type(kg_step_stats) :: stats
      end function
      integer(c_int) function kg_hydraulic_rhs(ctx, t, substep, advised_dt) bind(C, name="kg_hydraulic_rhs")
         import :: c_int, c_int32_t, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double), value :: t
         integer(c_int32_t), value :: substep
         real(c_double) :: advised_dt
      end function
      integer(c_int) function kg_get_active_tiles(ctx, ids, n) bind(C, name="kg_get_active_tiles")
         import :: c_int, c_int32_t, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int32_t) :: ids(*)
         integer(c_int32_t) :: n                ! capacity on entry, count on exit
      end function
      integer(c_int) function kg_set_tile_field(ctx, tile, field, in) bind(C, name="kg_set_tile_field")
         import :: c_int, c_int32_t, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: tile, field
         real(c_double), intent(in) :: in(*)
      end function
      integer(c_int) function kg_get_tile_vertex(ctx, tile, which, out) bind(C, name="kg_get_tile_vertex")
         import :: c_int, c_int32_t, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: tile, which   ! 0: b0, 1: bt
         real(c_double) :: out(*)
      end function
      integer(c_int) function kg_get_tile_rhs(ctx, tile, k, out) bind(C, name="kg_get_tile_rhs")
         import :: c_int, c_int32_t, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: tile, k       ! 1..4: ddtExplicit rows, 5: ddtImplicit
         real(c_double) :: out(*)
      end function
      integer(c_int) function kg_get_tile_maxima(ctx, tile, which, out) bind(C, name="kg_get_tile_maxima")
         import :: c_int, c_int32_t, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: tile, which   ! 0..4: (value, time) of Hn, u, e, d, psi; 5: tfirst
         real(c_double) :: out(*)
      end function
      integer(c_int) function kg_get_state(ctx, ids, n, state, bt_vertex) bind(C, name="kg_get_state")
         import :: c_int, c_int32_t, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t) :: ids(*)
         integer(c_int32_t) :: n                ! capacity on entry, count on exit
         real(c_double) :: state(*)             ! (nX, nY, 4, n) in Fortran order
         real(c_double) :: bt_vertex(*)         ! (nX+1, nY+1, n)
      end function
      integer(c_int) function kg_load_state(ctx, ids, n, state, bt_vertex, t) bind(C, name="kg_load_state")
         import :: c_int, c_int32_t, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int32_t), intent(in) :: ids(*)
         integer(c_int32_t), value :: n
         real(c_double), intent(in) :: state(*)
         real(c_double), intent(in) :: bt_vertex(*)
         real(c_double), value :: t
      end function
      integer(c_int) function kg_get_time(ctx, t, dt) bind(C, name="kg_get_time")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double) :: t, dt
      end function
      ! FP32 form: each morphodynamic stage as one launch (1, default) or three (0)
      integer(c_int) function kg_set_fused_morpho(ctx, enable) bind(C, name="kg_set_fused_morpho")
         import :: c_int, c_int32_t, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: enable
      end function
      ! FP32 form: skip the flux work of blocks with no water (1, default) or not (0)
      integer(c_int) function kg_set_dry_skip(ctx, enable) bind(C, name="kg_set_dry_skip")
         import :: c_int, c_int32_t, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int32_t), value :: enable
      end function
      subroutine kg_destroy(ctx) bind(C, name="kg_destroy")
         import :: c_ptr
         type(c_ptr), value :: ctx
      end subroutine
      type(c_ptr) function kg_last_error(ctx) bind(C, name="kg_last_error")
         import :: c_ptr
         type(c_ptr), value :: ctx             ! c_null_ptr: why the last kg_create failed
      end function
   end interface
contains
   ! A nonzero status becomes the reference's fatal error (src/Messages.f90:56-90).
   subroutine kg_check(rc, ctx)
      use messages_module, only: FatalErrorMessage
      integer(c_int), intent(in) :: rc
      type(c_ptr), intent(in) :: ctx
      character(kind=c_char), pointer :: s(:)
      character(len=512) :: msg
      integer :: n
      if (rc == 0) return
      call c_f_pointer(kg_last_error(ctx), s, [512])
      msg = ''
      n = 0
      do while (n < 512)
         if (s(n + 1) == c_null_char) exit
         n = n + 1
         msg(n:n) = s(n)
      end do
      call FatalErrorMessage(msg(1:max(n, 1)))
   end subroutine
end module kestrel_gpu
