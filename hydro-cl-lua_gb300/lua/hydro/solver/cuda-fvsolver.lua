--[[
A 'cuda' finite-volume solver for hydro-cl-lua: same args table as
hydro/solver/fvsolver.lua (eqn='euler', flux='roe', 'hll', 'rusanov' or
'euler-hllc', coord='cartesian'), with the update -- boundary, calcLR ("plm
cons", "plm prim", "plm athena"), calcFlux,
calcDerivFromFlux,
the integrator's multAdd sequence, constrainU, calcDT -- run by libhydrocuda on
one GPU instead of by the OpenCL kernels.

	self.solvers:insert(require 'hydro.solver.cuda-fvsolver'(table(args, {
		flux = 'roe',
		eqn = 'euler',
		cudaPrecision = 'f64 plain',   -- or 'f64' / 'f32' for the fused forms
	})))

The class keeps FiniteVolumeSolver for everything around the update (display
variables, GUI, initial conditions, buffers), and replaces the update path:
after each resetState the OpenCL UBuf is copied into the CUDA solver; after
each update the CUDA state is copied back into UBuf (host round trip) only
when something reads it (display, save, calcExactError) -- see syncToCL.

Put this file on package.path as hydro/solver/cuda-fvsolver.lua inside the
reference checkout, and lua/hydrocuda_ffi.lua beside it (or on package.path).
--]]
local ffi = require 'ffi'
local table = require 'ext.table'
local FiniteVolumeSolver = require 'hydro.solver.fvsolver'
local hc = require 'hydrocuda_ffi'

local CudaFVSolver = FiniteVolumeSolver:subclass()
CudaFVSolver.name = 'cuda-fvsolver'

local sharedCtx

local function descFromSolver(self, args)
	assert(self.eqn.name == 'euler', "the cuda solver provides eqn='euler'")
	local flux = assert(hc.fluxIndex[self.flux.name], "the cuda solver provides flux='roe', 'hll', 'rusanov' and 'euler-hllc'")
	assert(require 'hydro.coord.cartesian':isa(self.coord), "the cuda solver provides coord='cartesian'")
	local d = ffi.new'hc_solver_desc'
	d.dim = self.dim
	for i=0,2 do
		d.n[i] = i < self.dim and tonumber(self.sizeWithoutBorder.s[i]) or 1
		d.mins[i] = self.mins.s[i]
		d.maxs[i] = self.maxs.s[i]
	end
	local k = 0
	for _,xi in ipairs{'x','y','z'} do
		for _,mm in ipairs{'min','max'} do
			local name = self.boundaryMethods[xi..mm].name
			d.boundary[k] = assert(hc.boundaryIndex[name],
				"the cuda solver provides none, periodic, mirror, freeflow, linear, quadratic and fixed boundaries")
			if name == 'fixed' then
				-- BoundaryFixed's fixedCode generates OpenCL; the library takes
				-- the constant state itself: args.cudaFixedCons[side] =
				-- {rho, m.x, m.y, m.z, ETotal}
				local c = assert((args.cudaFixedCons or {})[xi..mm],
					"a fixed boundary needs cudaFixedCons."..xi..mm.." = {rho, m.x, m.y, m.z, ETotal}")
				for f=0,4 do d.fixed_cons[k][f] = c[f+1] end
			end
			k = k + 1
		end
	end
	d.flux_limiter = self.fluxLimiter - 1
	d.recon = self.usePLM and assert(hc.reconIndex[self.usePLM], "the cuda solver provides usePLM='piecewise constant', 'plm cons', 'plm prim' and 'plm athena'") or 0
	d.slope_limiter = self.slopeLimiter - 1
	d.integrator = assert(hc.integratorIndex[self.integrator.name], "the cuda solver provides the explicit integrators")
	d.precision = hc.precisionIndex[args.cudaPrecision or 'f64 plain']
	local solverPtr = self.solverPtr
	d.gamma = solverPtr.heatCapacityRatio
	d.rho_min = solverPtr.rhoMin
	d.p_min = solverPtr.PMin
	d.cfl = self.cfl
	d.fixed_dt = self.useFixedDT and self.fixedDT or 0
	d.flux = flux
	d.hllc_method = self.flux.hllcMethod and (self.flux.hllcMethod + 1) or 0
	-- Roe's useEntropyFluxFix (hydro/flux/roe.lua:10-16)
	d.entropy_fix = self.flux.useEntropyFluxFix and 1 or 0
	d.entropy_fix_factor = self.flux.entropyFluxFixLimitingFactor or .2
	return d
end

function CudaFVSolver:init(args)
	CudaFVSolver.super.init(self, args)
	if not sharedCtx then
		local p = ffi.new'hc_context*[1]'
		hc.check(hc.lib.hc_context_create(args.cudaDevice or 0, p))
		sharedCtx = p[0]
	end
	local p = ffi.new'hc_solver*[1]'
	local desc = descFromSolver(self, args)
	hc.check(hc.lib.hc_solver_create(sharedCtx, desc, p))
	self.hcSolver = ffi.gc(p[0], hc.lib.hc_solver_destroy)
	self.hcPlain = desc.precision == 0
	self.hcNeedsUpload = true
	-- the fused forms pick their fastest stage-kernel schedule for this grid
	-- once the state is set (cudaAutotune = false keeps the default one)
	self.hcAutotune = not self.hcPlain and args.cudaAutotune ~= false
end

-- The update's OpenCL kernels (calcLR, calcFlux, calcDerivFromFlux) are
-- replaced by libhydrocuda, so their modules leave the solver program: they
-- are neither generated nor compiled (SolverBase:refreshSolverProgram,
-- solverbase.lua:1670-1735, builds the program from solverModulesEnabled;
-- fvsolver.lua:41,49 and gridsolver.lua:351 add these three).  The rest --
-- display variables, boundary, constrainU, calcDT -- stays for the OpenCL
-- side's own uses (display, GUI, the boundary fill before the first upload).
function CudaFVSolver:initCodeModules()
	CudaFVSolver.super.initCodeModules(self)
	for _,name in ipairs{'calcLR', 'calcFlux', 'calcDerivFromFlux'} do
		local sym = self.symbols[name]
		if sym then self.solverModulesEnabled[sym] = nil end
	end
end

-- SolverBase's program build only: the GridSolver and FiniteVolumeSolver
-- overrides (gridsolver.lua:444-456, fvsolver.lua:213-222) would look up the
-- kernels left out above
function CudaFVSolver:refreshSolverProgram()
	require 'hydro.solver.solverbase'.refreshSolverProgram(self)
end

-- whole UBuf (ghosts included) between the OpenCL buffer and the CUDA solver;
-- real must be double for the plain form's ghost-inclusive I/O
local function ubufHost(self)
	assert(ffi.sizeof'real' == 8, "the cuda solver exchanges UBuf in real=double")
	return ffi.cast('double*', self.UBufObj:toCPU())
end

-- interior cell k (x-fastest) <-> UBuf index with numGhost layers
local function forInterior(self, f)
	local G = self.numGhost
	local n = {}
	for i=0,2 do n[i] = i < self.dim and tonumber(self.sizeWithoutBorder.s[i]) or 1 end
	local sx, sy = tonumber(self.gridSize.x), tonumber(self.gridSize.y)
	local k = 0
	for z=0,n[2]-1 do
		for y=0,n[1]-1 do
			for x=0,n[0]-1 do
				local gx = x + G
				local gy = self.dim > 1 and y + G or y
				local gz = self.dim > 2 and z + G or z
				f(k, gx + sx * (gy + sy * gz))
				k = k + 1
			end
		end
	end
	return k
end

function CudaFVSolver:syncFromCL()
	local ptr = ubufHost(self)
	if self.hcPlain then
		-- the plain form keeps the reference's whole UBuf, ghosts included
		hc.check(hc.lib.hc_solver_set_state(self.hcSolver, ptr, hc.LAYOUT_AOS6_F64, 1))
	else
		local interior = ffi.new('double[?]', tonumber(self.numCells) * 6)
		forInterior(self, function(k, i)
			for j=0,5 do interior[6*k+j] = ptr[6*i+j] end
		end)
		hc.check(hc.lib.hc_solver_set_state(self.hcSolver, interior, hc.LAYOUT_AOS6_F64, 0))
	end
	self.hcNeedsUpload = false
end

function CudaFVSolver:syncToCL()
	local n = tonumber(self.numCells)
	local buf = ffi.new('double[?]', n * 6)
	if self.hcPlain then
		hc.check(hc.lib.hc_solver_get_state(self.hcSolver, buf, hc.LAYOUT_AOS6_F64, 1))
	else
		local full = ubufHost(self)
		local interior = ffi.new('double[?]', n * 6)
		hc.check(hc.lib.hc_solver_get_state(self.hcSolver, interior, hc.LAYOUT_AOS6_F64, 0))
		ffi.copy(buf, full, n * 6 * 8)
		forInterior(self, function(k, i)
			for j=0,5 do buf[6*i+j] = interior[6*k+j] end
		end)
	end
	self.UBufObj:fromCPU(buf)
	-- the ghost layers follow from the interior
	CudaFVSolver.super.boundary(self)
end

function CudaFVSolver:resetState()
	CudaFVSolver.super.resetState(self)
	self:syncFromCL()
	hc.check(hc.lib.hc_solver_set_time(self.hcSolver, 0))
	if self.hcAutotune then
		-- leaves the state and time as they are
		hc.check(hc.lib.hc_solver_autotune(self.hcSolver, nil))
		self.hcAutotune = false
	end
end

function CudaFVSolver:boundary()
	if self.hcSolver and not self.hcNeedsUpload then
		hc.check(hc.lib.hc_solver_boundary(self.hcSolver))
	else
		CudaFVSolver.super.boundary(self)
	end
end

function CudaFVSolver:constrainU()
	if self.hcSolver and not self.hcNeedsUpload then
		hc.check(hc.lib.hc_solver_constrain_u(self.hcSolver))
	else
		CudaFVSolver.super.constrainU(self)
	end
end

function CudaFVSolver:calcDT()
	if self.hcNeedsUpload then self:syncFromCL() end
	local dt = ffi.new'double[1]'
	hc.check(hc.lib.hc_solver_calc_dt(self.hcSolver, dt))
	self.fixedDT = dt[0]
	return dt[0]
end

function CudaFVSolver:step(dt)
	if self.hcNeedsUpload then self:syncFromCL() end
	hc.check(hc.lib.hc_solver_step(self.hcSolver, dt))
end

-- SolverBase:update (solverbase.lua:3026-3190) without the console/trackvars
-- block: calcDT, step, t += dt, boundary -- one library call.
function CudaFVSolver:update()
	if self.hcNeedsUpload then self:syncFromCL() end
	local dt = ffi.new'double[1]'
	hc.check(hc.lib.hc_solver_update(self.hcSolver, dt))
	self.t = self.t + dt[0]
	self.dt = dt[0]
	self.solverPtr.t = self.t
	self.solverPtr.dt = self.dt
	self:refreshSolverBuf()
	self.hcStateOnGPUOnly = true
end

-- anything that reads UBuf on the OpenCL side (display vars, save,
-- calcExactError) first pulls the state back
function CudaFVSolver:calcDisplayVarToTex(...)
	if self.hcStateOnGPUOnly then self:syncToCL() self.hcStateOnGPUOnly = false end
	return CudaFVSolver.super.calcDisplayVarToTex(self, ...)
end

function CudaFVSolver:calcExactError(...)
	if self.hcStateOnGPUOnly then self:syncToCL() self.hcStateOnGPUOnly = false end
	return CudaFVSolver.super.calcExactError(self, ...)
end

function CudaFVSolver:save(...)
	if self.hcStateOnGPUOnly then self:syncToCL() self.hcStateOnGPUOnly = false end
	return CudaFVSolver.super.save(self, ...)
end

return CudaFVSolver
