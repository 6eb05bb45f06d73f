! kestrel_gpu_dropin.f90 -- the GB300 hot path behind the reference's own module interfaces.
!
! timestepper_gpu_module offers the public procedures of timestepper_module
! (src/TimeStepper.f90:64, :73, :116) and hydraulic_rhs_module (src/HydraulicRHS.f90:41,
! :64-73) with the same argument lists, so that the host switches to the GPU path by
! changing one use statement in src/main.f90:50:
!
!    use timestepper_gpu_module, only: Run
!
! and keeps everything else: input parsing, InitialiseGrid, LoadDEM, LoadSourceConditions
! and the output writers run unchanged on the host grid.  The run settings are copied
! field by field into kg_params (MakeKgParams), the closure, limiter, boundary and
! topography names the input parser stores (src/Parameters.f90:171-466,
! src/SolverSettings.f90:102-126, src/TopogSettings.f90:125-140) become the header's
! selector values, and after every IntegrateTo the GPU state is mirrored into
! grid%tileContainer (tiles the GPU activated are added on the host with the reference's
! own AddTile first), so that OutputSolutionData, CalculateVolume and OutputAggregateData
! read what they read from the reference's stepper.  Every status goes through kg_check
! (a nonzero code becomes FatalErrorMessage).
!
! Analytic topography (Topog = Function) is built on the device from the same parameters.
! For a raster (Topog = Raster/DEM) the host hands the GDAL values of DEM.vrt and its
! geotransform to SetRaster before the first IntegrateTo (kg_upload_raster).
module timestepper_gpu_module
   use, intrinsic :: iso_c_binding
   use set_precision_module, only: wp
   use runsettings_module, only: RunSet
   use grid_module, only: GridType, TileType
   use update_tiles_module, only: AddTile
   use output_module, only: OutputSolutionData, OutputInfo, CalculateVolume, OutputAggregateData
   use messages_module, only: FatalErrorMessage
   use varstring_module, only: varString
   use kestrel_gpu
   implicit none

   private
   public :: Run, IntegrateTo, CalculateHydraulicRHS, MakeKgParams, SetRaster, SetPrecisionForm

   type(c_ptr), save :: ctx = c_null_ptr
   integer(c_int32_t), save :: precision_form = 0_c_int32_t   ! 0: FP64 plain, 1: the FP32 form
   logical, save :: have_raster = .false.
   real(c_double), allocatable, target, save :: raster_values(:)
   type(kg_raster), save :: raster_geo

contains

   ! 0 selects the FP64 plain path (the drop-in), 1 the FP32 form.  Call before Run.
   subroutine SetPrecisionForm(form)
      integer, intent(in) :: form
      precision_form = int(form, c_int32_t)
   end subroutine SetPrecisionForm

   ! Raster topography for the device: values in RasterIO order (rows from the north, x
   ! fastest) and the geotransform GDAL returns for DEM.vrt (src/dem.f90:203-356), with the
   ! projected domain centre (RunParams%centerUTM).
   subroutine SetRaster(values, geo)
      real(c_double), intent(in) :: values(:)
      type(kg_raster), intent(in) :: geo
      raster_values = values
      raster_geo = geo
      have_raster = .true.
   end subroutine SetRaster

   ! Index of name in the list (case-insensitive), or -1.
   integer function pick(name, names) result(k)
      character(len=*), intent(in) :: name
      character(len=*), intent(in) :: names(:)
      integer :: i
      k = -1
      do i = 1, size(names)
         if (lower(trim(name)) == lower(trim(names(i)))) then
            k = i - 1
            return
         end if
      end do
   end function pick

   function lower(s) result(t)
      character(len=*), intent(in) :: s
      character(len=len(s)) :: t
      integer :: i, c
      t = s
      do i = 1, len(s)
         c = iachar(s(i:i))
         if (c >= iachar('A') .and. c <= iachar('Z')) t(i:i) = achar(c + 32)
      end do
   end function lower

   integer(c_int32_t) function shape_id(shape) result(k)
      character(len=*), intent(in) :: shape
      k = int(max(0, pick(shape, [character(len=8) :: 'flat', 'para', 'level'])), c_int32_t)
   end function shape_id

   ! RunSet (src/RunSettings.f90:161-340) -> kg_params, field by field.
   subroutine MakeKgParams(RunParams, p)
      type(RunSet), intent(in) :: RunParams
      type(kg_params), intent(out) :: p
      integer :: k, n

      p%nXtiles = RunParams%nXtiles
      p%nYtiles = RunParams%nYtiles
      p%nXpertile = RunParams%nXpertile
      p%nYpertile = RunParams%nYpertile
      p%Xtilesize = RunParams%Xtilesize
      p%Ytilesize = RunParams%Ytilesize
      p%bcs = int(pick(RunParams%bcs%s, [character(len=10) :: 'halt', 'periodic', 'dirichlet', 'sponge']), c_int32_t)
      p%pad0 = 0
      p%bcsHnval = RunParams%bcsHnval
      p%bcsuval = RunParams%bcsuval
      p%bcsvval = RunParams%bcsvval
      p%bcspsival = RunParams%bcspsival
      p%geometric_factors = merge(1_c_int32_t, 0_c_int32_t, RunParams%geometric_factors)
      p%MorphodynamicsOn = merge(1_c_int32_t, 0_c_int32_t, RunParams%MorphodynamicsOn)
      p%g = RunParams%g
      p%rhow = RunParams%rhow
      p%rhos = RunParams%rhos
      p%ChezyCo = RunParams%ChezyCo
      p%ManningCo = RunParams%ManningCo
      p%CoulombCo = RunParams%CoulombCo
      p%PouliquenMinSlope = RunParams%PouliquenMinSlope
      p%PouliquenMaxSlope = RunParams%PouliquenMaxSlope
      p%PouliquenIntermediateSlope = RunParams%PouliquenIntermediateSlope
      p%PouliquenBeta = RunParams%PouliquenBeta
      p%Edwards2019betastar = RunParams%Edwards2019betastar
      p%Edwards2019kappa = RunParams%Edwards2019kappa
      p%Edwards2019Gamma = RunParams%Edwards2019Gamma
      p%VoellmySwitchRate = RunParams%VoellmySwitchRate
      p%VoellmySwitchValue = RunParams%VoellmySwitchValue
      p%EroRate = RunParams%EroRate
      p%EroRateGranular = RunParams%EroRateGranular
      p%EroDepth = RunParams%EroDepth
      p%EroCriticalHeight = RunParams%EroCriticalHeight
      p%BedPorosity = RunParams%BedPorosity
      p%maxPack = RunParams%maxPack
      p%SolidDiameter = RunParams%SolidDiameter
      p%EddyViscosity = RunParams%EddyViscosity
      ! the settling speed as the reference derived it (src/Parameters.f90:629-648)
      p%ws0_given = 1
      p%pad1 = 0
      p%ws0 = RunParams%ws0
      p%drag = int(pick(RunParams%DragChoice%s, [character(len=12) :: 'chezy', 'coulomb', 'voellmy', 'pouliquen', &
                                                  'edwards2019', 'variable', 'manning']), c_int32_t)
      p%erosion = int(max(0, pick(RunParams%ErosionChoice%s, [character(len=10) :: 'off', 'mixed', 'simple', 'fluid', &
                                                                'granular'])), c_int32_t)
      if (.not. RunParams%MorphodynamicsOn) p%erosion = 0
      p%deposition = int(pick(RunParams%DepositionChoice%s, [character(len=16) :: 'none', 'simple', &
                                                               'spearman manning']), c_int32_t)
      p%erosion_transition = int(pick(RunParams%ErosionTransition%s, [character(len=8) :: 'smooth', 'step', 'off']), &
                                 c_int32_t)
      p%morpho_damping = int(pick(RunParams%MorphoDamp%s, [character(len=8) :: 'none', 'tanh', 'rat3']), c_int32_t)
      p%fswitch = int(pick(RunParams%fswitch%s, [character(len=8) :: 'tanh', 'rat3', 'cos', 'linear', 'equal', 'zero', &
                                                  'one', 'step']), c_int32_t)
      p%limiter = int(pick(RunParams%limiter%s, [character(len=10) :: 'minmod1', 'minmod2', 'van albada', 'weno', &
                                                  'none']), c_int32_t)
      p%TileBuffer = RunParams%TileBuffer
      p%heightThreshold = RunParams%heightThreshold
      p%cfl = RunParams%cfl
      p%maxdt = RunParams%maxdt
      p%tstart = RunParams%tstart
      p%tend = RunParams%tend
      p%SpongeStrength = RunParams%SpongeStrength
      p%Nout = RunParams%Nout
      p%pad2 = 0
      p%nCaps = 0
      p%nCubes = 0
      p%nSources = 0
      p%pad3 = 0
      ! Sources were already placed on the host by LoadSourceConditions; the device places
      ! them again from the same settings (kg_load_sources).
      if (RunParams%set_Caps) then
         p%nCaps = min(RunParams%nCaps, size(p%caps))
         do k = 1, p%nCaps
            p%caps(k)%x = RunParams%CapSources(k)%x
            p%caps(k)%y = RunParams%CapSources(k)%y
            p%caps(k)%radius = RunParams%CapSources(k)%radius
            p%caps(k)%height = RunParams%CapSources(k)%height
            p%caps(k)%psi = RunParams%CapSources(k)%psi
            p%caps(k)%u = RunParams%CapSources(k)%u
            p%caps(k)%v = RunParams%CapSources(k)%v
            p%caps(k)%shape = shape_id(RunParams%CapSources(k)%shape)
            p%caps(k)%pad = 0
         end do
      end if
      if (RunParams%set_Cubes) then
         p%nCubes = min(RunParams%nCubes, size(p%cubes))
         do k = 1, p%nCubes
            p%cubes(k)%x = RunParams%CubeSources(k)%x
            p%cubes(k)%y = RunParams%CubeSources(k)%y
            p%cubes(k)%length = RunParams%CubeSources(k)%length
            p%cubes(k)%width = RunParams%CubeSources(k)%width
            p%cubes(k)%height = RunParams%CubeSources(k)%height
            p%cubes(k)%psi = RunParams%CubeSources(k)%psi
            p%cubes(k)%u = RunParams%CubeSources(k)%u
            p%cubes(k)%v = RunParams%CubeSources(k)%v
            p%cubes(k)%shape = shape_id(RunParams%CubeSources(k)%shape)
            p%cubes(k)%pad = 0
         end do
      end if
      if (RunParams%set_Sources) then
         p%nSources = min(RunParams%nSources, size(p%sources))
         do k = 1, p%nSources
            n = min(size(RunParams%FluxSources(k)%time), size(p%sources(k)%time))
            p%sources(k)%x = RunParams%FluxSources(k)%x
            p%sources(k)%y = RunParams%FluxSources(k)%y
            p%sources(k)%radius = RunParams%FluxSources(k)%radius
            p%sources(k)%n_series = n
            p%sources(k)%pad = 0
            p%sources(k)%time(1:n) = RunParams%FluxSources(k)%time(1:n)
            p%sources(k)%flux(1:n) = RunParams%FluxSources(k)%flux(1:n)
            p%sources(k)%psi(1:n) = RunParams%FluxSources(k)%psi(1:n)
         end do
      end if
      p%n_topog_params = 0
      p%topog_params = 0.0_c_double
      select case (lower(RunParams%Topog%s))
      case ('function')
         p%topog = int(pick(RunParams%TopogFunc%s, [character(len=20) :: 'upload', 'flat', 'xslope', 'yslope', &
                       'xyslope', 'xsinslope', 'xysinslope', 'xhump', 'xtanh', 'xparab', 'xyparab', 'raster', &
                       'x2slopes', 'usgs', 'flume', 'channel power law', 'channel trapezium', 'xbislope', &
                       'xtrislope']), c_int32_t)
         if (allocated(RunParams%TopogFuncParams)) then
            p%n_topog_params = int(min(size(RunParams%TopogFuncParams), size(p%topog_params)), c_int32_t)
            p%topog_params(1:p%n_topog_params) = RunParams%TopogFuncParams(1:p%n_topog_params)
         end if
      case default
         p%topog = 11   ! KG_TOPO_RASTER: the values come from SetRaster
      end select
   end subroutine MakeKgParams

   ! The device context of this run, created on first use from RunParams.
   subroutine EnsureContext(RunParams)
      type(RunSet), intent(in) :: RunParams
      type(kg_params), target, save :: p
      if (c_associated(ctx)) return
      call MakeKgParams(RunParams, p)
      call kg_check(kg_create(c_loc(p), precision_form, ctx), c_null_ptr)
      if (p%topog == 11) then
         if (.not. have_raster) call FatalErrorMessage("Error: raster topography needs SetRaster before the first step.")
         call kg_check(kg_upload_raster(ctx, raster_values, raster_geo), ctx)
      end if
      call kg_check(kg_load_sources(ctx), ctx)
   end subroutine EnsureContext

   ! Run (src/TimeStepper.f90:73-112): the same output schedule, IntegrateTo on the GPU.
   subroutine Run(RunParams, grid)
      type(RunSet), intent(inout) :: RunParams
      type(GridType), target, intent(inout) :: grid
      real(kind=wp) :: timestep
      integer :: i

      RunParams%CurrentOut = RunParams%FirstOut
      if (.not. RunParams%Restart) then
         call OutputSolutionData(RunParams, RunParams%CurrentOut, grid)
         call OutputInfo(RunParams)
         call CalculateVolume(RunParams, RunParams%tstart, grid, create = .true.)
      end if
      do i = 1, RunParams%Nout - RunParams%FirstOut
         timestep = RunParams%tstart + (i + RunParams%FirstOut) * RunParams%DeltaT
         call IntegrateTo(RunParams, timestep, grid)
         RunParams%CurrentOut = RunParams%CurrentOut + 1
         call OutputSolutionData(RunParams, RunParams%CurrentOut, grid)
         call CalculateVolume(RunParams, timestep, grid)
         call OutputAggregateData(RunParams, grid)
         call OutputInfo(RunParams)
      end do
      call kg_destroy(ctx)
      ctx = c_null_ptr
   end subroutine Run

   ! IntegrateTo (src/TimeStepper.f90:116-277): the device integrates to tend, then the
   ! host grid receives the state its writers read.
   subroutine IntegrateTo(RunParams, tend, grid)
      type(RunSet), intent(inout) :: RunParams
      real(kind=wp), intent(in) :: tend
      type(GridType), target, intent(inout) :: grid
      type(kg_step_stats) :: stats

      call EnsureContext(RunParams)
      call kg_check(kg_integrate_to(ctx, real(tend, c_double), stats), ctx)
      call MirrorState(RunParams, grid)
   end subroutine IntegrateTo

   ! CalculateHydraulicRHS (src/HydraulicRHS.f90:64-136) on the device: the solution of the
   ! active tiles of tileWorkspace goes up, ddtExplicit / ddtImplicit come back, and the
   ! advised time step is the device's.  The device's active set is the host's (both grow
   ! only through the steps above).
   subroutine CalculateHydraulicRHS(RunParams, grid, tileWorkspace, t, substep, advisedTimeStep)
      type(RunSet), intent(in) :: RunParams
      type(GridType), target, intent(inout) :: grid
      type(TileType), dimension(:), intent(inout) :: tileWorkspace
      real(kind=wp), intent(in) :: t
      integer, intent(in) :: substep
      real(kind=wp), intent(out) :: advisedTimeStep
      real(c_double), allocatable :: plane(:)
      real(c_double) :: adv
      integer :: tt, ttk, f, nX, nY

      call EnsureContext(RunParams)
      nX = RunParams%nXpertile
      nY = RunParams%nYpertile
      allocate (plane(nX * nY))
      do tt = 1, grid%activeTiles%size
         ttk = grid%activeTiles%List(tt)
         do f = 1, 4
            plane = reshape(tileWorkspace(ttk)%u(f, :, :), [nX * nY])
            call kg_check(kg_set_tile_field(ctx, int(ttk, c_int32_t), int(f, c_int32_t), plane), ctx)
         end do
      end do
      call kg_check(kg_hydraulic_rhs(ctx, real(t, c_double), int(substep, c_int32_t), adv), ctx)
      advisedTimeStep = adv
      do tt = 1, grid%activeTiles%size
         ttk = grid%activeTiles%List(tt)
         do f = 1, 4
            call kg_check(kg_get_tile_rhs(ctx, int(ttk, c_int32_t), int(f, c_int32_t), plane), ctx)
            tileWorkspace(ttk)%ddtExplicit(f, :, :) = reshape(plane, [nX, nY])
         end do
         call kg_check(kg_get_tile_rhs(ctx, int(ttk, c_int32_t), 5_c_int32_t, plane), ctx)
         tileWorkspace(ttk)%ddtImplicit(:, :, :) = 0.0_wp
         tileWorkspace(ttk)%ddtImplicit(2, :, :) = reshape(plane, [nX, nY])
         tileWorkspace(ttk)%ddtImplicit(3, :, :) = reshape(plane, [nX, nY])
      end do
   end subroutine CalculateHydraulicRHS

   ! The device state into grid%tileContainer: tiles the device activated are added on the
   ! host (AddTile, src/UpdateTiles.f90:56-78, which also adds their ghost tiles), then the
   ! 13 fields, the vertex bed change and the running maxima of every active tile, and the
   ! clock.
   subroutine MirrorState(RunParams, grid)
      type(RunSet), intent(in) :: RunParams
      type(GridType), target, intent(inout) :: grid
      integer(c_int32_t), allocatable :: ids(:)
      real(c_double), allocatable :: plane(:), vert(:), mx(:)
      integer(c_int32_t) :: n
      real(c_double) :: t, dt
      integer :: k, f, id, nX, nY

      nX = RunParams%nXpertile
      nY = RunParams%nYpertile
      n = 0
      call kg_check(kg_get_active_tiles(ctx, ids_dummy(), n), ctx)
      allocate (ids(max(n, 1)))
      call kg_check(kg_get_active_tiles(ctx, ids, n), ctx)
      allocate (plane(nX * nY), vert((nX + 1) * (nY + 1)), mx(2 * nX * nY))
      do k = 1, n
         id = ids(k)
         if (.not. any(grid%activeTiles%List(1:grid%activeTiles%size) == id)) call AddTile(grid, id, RunParams)
         do f = 1, 13
            call kg_check(kg_get_tile_field(ctx, int(id, c_int32_t), int(f, c_int32_t), plane), ctx)
            grid%tileContainer(id)%u(f, :, :) = reshape(plane, [nX, nY])
         end do
         call kg_check(kg_get_tile_vertex(ctx, int(id, c_int32_t), 1_c_int32_t, vert), ctx)
         grid%tileContainer(id)%bt(:, :) = reshape(vert, [nX + 1, nY + 1])
         call MirrorMaxima(grid%tileContainer(id), int(id, c_int32_t), nX, nY, mx, plane)
      end do
      call kg_check(kg_get_time(ctx, t, dt), ctx)
      grid%t = t
      grid%dt = dt
   end subroutine MirrorState

   subroutine MirrorMaxima(tile, id, nX, nY, mx, plane)
      type(TileType), intent(inout) :: tile
      integer(c_int32_t), intent(in) :: id
      integer, intent(in) :: nX, nY
      real(c_double), intent(inout) :: mx(:), plane(:)
      call kg_check(kg_get_tile_maxima(ctx, id, 0_c_int32_t, mx), ctx)
      if (allocated(tile%Hnmax)) tile%Hnmax = reshape(mx, [nX, nY, 2])
      call kg_check(kg_get_tile_maxima(ctx, id, 1_c_int32_t, mx), ctx)
      if (allocated(tile%umax)) tile%umax = reshape(mx, [nX, nY, 2])
      call kg_check(kg_get_tile_maxima(ctx, id, 2_c_int32_t, mx), ctx)
      if (allocated(tile%emax)) tile%emax = reshape(mx, [nX, nY, 2])
      call kg_check(kg_get_tile_maxima(ctx, id, 3_c_int32_t, mx), ctx)
      if (allocated(tile%dmax)) tile%dmax = reshape(mx, [nX, nY, 2])
      call kg_check(kg_get_tile_maxima(ctx, id, 4_c_int32_t, mx), ctx)
      if (allocated(tile%psimax)) tile%psimax = reshape(mx, [nX, nY, 2])
      call kg_check(kg_get_tile_maxima(ctx, id, 5_c_int32_t, plane), ctx)
      if (allocated(tile%tfirst)) tile%tfirst = reshape(plane, [nX, nY])
   end subroutine MirrorMaxima

   ! A one-element id buffer for the count-only query of kg_get_active_tiles (n = 0 on entry).
   function ids_dummy() result(a)
      integer(c_int32_t) :: a(1)
      a = 0
   end function ids_dummy

end module timestepper_gpu_module
