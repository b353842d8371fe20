--[[
Continuous-batching request loop over libhydrocuda's batch (hc_batch_*), the
Lua counterpart of serve.py with the same policy:

* arrived requests are offered for admission in arrival order against the
  batch's HBM budget and slot table; one that does not fit is passed over for
  now so smaller ones behind it start, unless it has waited longer than
  ageCap seconds -- then admission stops at it until retirements free enough
  memory, so a large request is not starved (at most maxRefusals refusals per
  pass);
* each tick queues stepsPerTick updates of every live solve
  (hc_batch_step_async), admits while they run, waits (hc_batch_wait), then
  polls the finished solves, fetches the kept results and retires their slots.

The reference has no serving layer: each hydro-cl-lua App steps its solvers in
its own loop (hydro/app.lua:1573-1750).  One request here is one App run to
exitTime.

	local hc = require 'hydrocuda_ffi'
	local serve = require 'hydro.serve'
	local batch = serve.Batch(ctx, {precision='f32', usePLM='plm cons', slopeLimiter='minmod',
		integrator='Runge-Kutta 2', maxSlots=1024, hbmBudget=150*2^30})
	local done = serve.Server{batch=batch, stepsPerTick=8}:run(requests)

A request is {arrival=seconds, desc=hc_solver_desc, init={kind='sod'|..., p={...}} or
cons=<double* AoS-6 interior state>, tEnd=t, tag=n, keep=bool}; finished requests come back
with admitted, finished, steps, t, status (and result, a double array, when keep is set).
--]]
local ffi = require 'ffi'
local hc = require 'hydrocuda_ffi'

ffi.cdef[[
typedef struct hc_serve_timespec { long tv_sec; long tv_nsec; } hc_serve_timespec;
int clock_gettime(int clk_id, hc_serve_timespec* tp);
int usleep(unsigned int usec);
]]

local M = {}

local CLOCK_MONOTONIC = 1
local function now()
	local ts = ffi.new'hc_serve_timespec'
	ffi.C.clock_gettime(CLOCK_MONOTONIC, ts)
	return tonumber(ts.tv_sec) + tonumber(ts.tv_nsec) * 1e-9
end
M.now = now

-- a batch of instances sharing one scheme (the keys of the reference's solver args)
local Batch = {}
Batch.__index = Batch

function M.Batch(ctx, args)
	local d = ffi.new'hc_batch_desc'
	d.precision = assert(hc.precisionIndex[args.precision or 'f32'], 'precision')
	assert(d.precision ~= 0, "batches run the fused forms ('f64' or 'f32')")
	d.flux_limiter = hc.limiterIndex[args.fluxLimiter or 'donor cell']
	d.recon = args.usePLM and assert(hc.reconIndex[args.usePLM], 'usePLM') or 0
	d.slope_limiter = hc.limiterIndex[args.slopeLimiter or 'donor cell']
	d.integrator = assert(hc.integratorIndex[args.integrator or 'forward Euler'], 'integrator')
	d.max_slots = args.maxSlots or 1024
	d.hbm_budget = args.hbmBudget or 150 * 2^30
	d.flux = hc.fluxIndex[args.flux or 'roe']
	local p = ffi.new'hc_batch*[1]'
	hc.check(hc.lib.hc_batch_create(ctx, d, p))
	return setmetatable({h = ffi.gc(p[0], hc.lib.hc_batch_destroy), maxSlots = d.max_slots}, Batch)
end

-- the slot, or nil when the budget or the slot table refuses
function Batch:tryAdmit(r)
	local slot = ffi.new'int[1]'
	local code
	if r.init then
		local ic = ffi.new'hc_init'
		hc.check(hc.lib.hc_init_defaults(assert(hc.initKind[r.init.kind], 'init kind'), ic))
		for i, v in ipairs(r.init.p or {}) do ic.p[i - 1] = v end
		if r.init.seed then ic.seed = r.init.seed end
		code = hc.lib.hc_batch_admit_init(self.h, r.desc, ic, r.tEnd, 0, r.tag, slot)
	else
		code = hc.lib.hc_batch_admit(self.h, r.desc, r.cons, hc.LAYOUT_AOS6_F64, r.tEnd, 0, r.tag, slot)
	end
	if code == hc.ERR_BUDGET or code == hc.ERR_NO_SLOT then return nil end
	hc.check(code)
	return slot[0]
end

function Batch:stepAsync(n) hc.check(hc.lib.hc_batch_step_async(self.h, n)) end
function Batch:wait() hc.check(hc.lib.hc_batch_wait(self.h, nil)) end

function Batch:poll()
	local cap = self.maxSlots
	local out = ffi.new('hc_done[?]', cap)
	local n = ffi.new'int[1]'
	hc.check(hc.lib.hc_batch_poll(self.h, out, cap, n))
	local evs = {}
	for i = 0, n[0] - 1 do
		evs[#evs + 1] = {slot = out[i].slot, status = out[i].status, tag = tonumber(out[i].tag),
			steps = tonumber(out[i].steps), t = out[i].t}
	end
	return evs
end

function Batch:fetch(slot, cells)
	local buf = ffi.new('double[?]', cells * 6)
	hc.check(hc.lib.hc_batch_fetch(self.h, slot, buf, hc.LAYOUT_AOS6_F64))
	return buf
end

function Batch:retire(slot) hc.check(hc.lib.hc_batch_retire(self.h, slot)) end

local function interiorCells(desc)
	local n = 1
	for k = 0, desc.dim - 1 do n = n * desc.n[k] end
	return n
end

local Server = {}
Server.__index = Server

function M.Server(args)
	return setmetatable({
		batch = assert(args.batch, 'batch'),
		stepsPerTick = args.stepsPerTick or 8,
		ageCap = args.ageCap or 1.0,
		maxRefusals = args.maxRefusals or 8,
		ticks = 0,
		cellUpdates = 0,
		passedOver = 0,
	}, Server)
end

-- one admission pass; returns how many started
function Server:admit(waiting, live, byTag, clock)
	local i, refused, started = 1, 0, 0
	while i <= #waiting and refused < self.maxRefusals do
		local r = waiting[i]
		local slot = self.batch:tryAdmit(r)
		if not slot then
			if live + started == 0 then error('request '..r.tag..' does not fit an empty batch') end
			refused = refused + 1
			if clock() - r.arrival > self.ageCap then break end
			i = i + 1
		else
			table.remove(waiting, i)
			if i > 1 then self.passedOver = self.passedOver + 1 end
			r.admitted = clock()
			r.slot = slot
			byTag[r.tag] = r
			started = started + 1
		end
	end
	return started
end

-- serves `requests` (arrival times in seconds from the start); returns the
-- finished requests
function Server:run(requests, clock)
	local t0 = now()
	clock = clock or function() return now() - t0 end
	local pending = {}
	for _, r in ipairs(requests) do pending[#pending + 1] = r end
	table.sort(pending, function(a, b) return a.arrival < b.arrival end)
	local next, waiting, live, done, byTag = 1, {}, 0, {}, {}
	while next <= #pending or #waiting > 0 or live > 0 do
		local t = clock()
		while next <= #pending and pending[next].arrival <= t do
			waiting[#waiting + 1] = pending[next]
			next = next + 1
		end
		local ticking = live > 0
		if ticking then self.batch:stepAsync(self.stepsPerTick) end
		local started = self:admit(waiting, live, byTag, clock)
		if ticking then
			self.batch:wait()
			self.ticks = self.ticks + 1
			for _, ev in ipairs(self.batch:poll()) do
				local r = byTag[ev.tag]
				byTag[ev.tag] = nil
				r.steps, r.t, r.status = ev.steps, ev.t, ev.status
				if r.keep then r.result = self.batch:fetch(ev.slot, interiorCells(r.desc)) end
				self.batch:retire(ev.slot)
				r.finished = clock()
				self.cellUpdates = self.cellUpdates + r.steps * interiorCells(r.desc)
				live = live - 1
				done[#done + 1] = r
			end
		end
		live = live + started
		if not ticking and started == 0 and #waiting == 0 and next <= #pending then
			-- idle until the next arrival
			local wait = pending[next].arrival - clock()
			if wait > 0 then ffi.C.usleep(math.floor(math.min(wait, 1) * 1e6)) end
		end
	end
	return done
end

-- p50 / p99 time-to-solution (seconds from arrival)
function M.latency(done)
	local lat = {}
	for _, r in ipairs(done) do lat[#lat + 1] = r.finished - r.arrival end
	table.sort(lat)
	local function pct(q)
		if #lat == 0 then return nil end
		return lat[math.max(1, math.ceil(q / 100 * #lat))]
	end
	return {count = #lat, p50 = pct(50), p99 = pct(99)}
end

return M
