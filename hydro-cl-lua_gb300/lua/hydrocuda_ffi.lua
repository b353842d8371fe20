--[[
LuaJIT ffi binding of libhydrocuda.so: the declarations of include/hydrocuda.h
that the 'cuda' solver class and the request loop (hydro/serve.lua) use.  Load with

	local hc = require 'hydrocuda_ffi'

The library is looked up next to this file's package directory
(hydro-cl-lua_gb300/libhydrocuda.so), then on the system path.
--]]
local ffi = require 'ffi'

ffi.cdef[[
typedef struct hc_solver_desc {
	int dim;
	int n[3];
	double mins[3];
	double maxs[3];
	int boundary[6];
	int flux_limiter;
	int recon;
	int slope_limiter;
	int integrator;
	int precision;
	double gamma;
	double rho_min;
	double p_min;
	double cfl;
	double fixed_dt;
	int flux;
	int hllc_method;
	int entropy_fix;
	int reserved0;
	double entropy_fix_factor;
	double fixed_cons[6][5];
} hc_solver_desc;
typedef struct hc_context hc_context;
typedef struct hc_solver hc_solver;
const char* hc_version(void);
const char* hc_last_error(void);
int hc_context_create(int device, hc_context** out);
int hc_context_destroy(hc_context* ctx);
int hc_solver_create(hc_context* ctx, const hc_solver_desc* desc, hc_solver** out);
int hc_solver_destroy(hc_solver* s);
int hc_solver_reset_state(hc_solver* s, const void* cons, int layout);
int hc_solver_set_state(hc_solver* s, const void* cons, int layout, int with_ghosts);
int hc_solver_get_state(hc_solver* s, void* cons, int layout, int with_ghosts);
int hc_solver_boundary(hc_solver* s);
int hc_solver_constrain_u(hc_solver* s);
int hc_solver_calc_dt(hc_solver* s, double* dt);
int hc_solver_step(hc_solver* s, double dt);
int hc_solver_update(hc_solver* s, double* dt_out);
int hc_solver_autotune(hc_solver* s, const char* cache_path);
int hc_solver_run_until(hc_solver* s, double t_end, long long max_steps, long long* steps_done);
int hc_solver_get_time(hc_solver* s, double* t);
int hc_solver_set_time(hc_solver* s, double t);
int hc_solver_status(hc_solver* s);
typedef struct hc_render {
	int mode;
	int var;
	int width, height;
	int palette;
	int use_log;
	double value_min, value_max;
	double bbox[4];
	double slice_angle[4];
	double fixed_z;
	double eye[3];
	double fov_y;
	double alpha, alpha_gamma, num_isobars;
	int max_iter;
	int use_isobars, use_lighting;
	int lic_iter;
	int noise_size;
	int reserved;
	unsigned long long noise_seed;
	int slice_axis;
	int num_slices;
} hc_render;
int hc_solver_display(hc_solver* s, int var, int zero_border, double* out);
int hc_solver_display_range(hc_solver* s, int var, double out[4]);
int hc_render_defaults(int mode, hc_render* out);
int hc_solver_render(hc_solver* s, const hc_render* r, unsigned char* rgba);
typedef struct hc_init {
	int kind;
	int reserved;
	unsigned long long seed;
	double p[16];
} hc_init;
typedef struct hc_batch_desc {
	int precision;
	int flux_limiter;
	int recon;
	int slope_limiter;
	int integrator;
	int max_slots;
	size_t hbm_budget;
	int flux;
	int hllc_method;
} hc_batch_desc;
typedef struct hc_done {
	int slot;
	int status;
	unsigned long long tag;
	long long steps;
	double t;
} hc_done;
typedef struct hc_batch hc_batch;
int hc_init_defaults(int kind, hc_init* out);
int hc_batch_create(hc_context* ctx, const hc_batch_desc* desc, hc_batch** out);
int hc_batch_destroy(hc_batch* b);
int hc_batch_admit(hc_batch* b, const hc_solver_desc* desc, const void* cons, int layout, double t_end, long long max_steps, unsigned long long tag, int* slot);
int hc_batch_admit_init(hc_batch* b, const hc_solver_desc* desc, const hc_init* init, double t_end, long long max_steps, unsigned long long tag, int* slot);
int hc_batch_step(hc_batch* b, int steps, int* n_active);
int hc_batch_step_async(hc_batch* b, int steps);
int hc_batch_wait(hc_batch* b, int* n_active);
int hc_batch_poll(hc_batch* b, hc_done* out, int cap, int* n_out);
int hc_batch_list(hc_batch* b, hc_done* out, int cap, int* n_out);
int hc_batch_fetch(hc_batch* b, int slot, void* cons, int layout);
int hc_batch_retire(hc_batch* b, int slot);
int hc_batch_autotune(hc_batch* b, const char* cache_path);
int hc_batch_set_schedule(hc_batch* b, int dim, int variant);
]]

local here = debug.getinfo(1, 'S').source:match'^@(.*)/[^/]*$' or '.'
local ok, lib = pcall(ffi.load, here .. '/../libhydrocuda.so')
if not ok then lib = ffi.load'hydrocuda' end

local M = {lib = lib}

-- names as in hydro/app.lua:614-635 (0-based for the C ABI)
M.limiterIndex = {}
for i, name in ipairs{
	'donor cell', 'Lax-Wendroff', 'Beam-Warming', 'Fromm', 'CHARM', 'HCUS', 'HQUICK', 'Koren',
	'minmod', 'Oshker', 'ospre', 'smart', 'Sweby', 'UMIST', 'van Albada 1', 'van Albada 2',
	'van Leer', 'monotized central', 'superbee', 'Barth-Jespersen', 'van Leer (abs)',
} do M.limiterIndex[name] = i - 1 end

M.integratorIndex = {}
for i, name in ipairs{
	'forward Euler', 'Runge-Kutta 2', 'Runge-Kutta 2 Heun', 'Runge-Kutta 2 Ralston', 'Runge-Kutta 3',
	'Runge-Kutta 4', 'Runge-Kutta 4, 3/8ths rule', 'Runge-Kutta 2, TVD', 'Runge-Kutta 2, non-TVD',
	'Runge-Kutta 3, TVD', 'Runge-Kutta 4, TVD', 'Runge-Kutta 4, non-TVD',
} do M.integratorIndex[name] = i - 1 end

M.boundaryIndex = {none = 0, periodic = 1, mirror = 2, freeflow = 3, linear = 4, quadratic = 5, fixed = 6}
M.fluxIndex = {roe = 0, hll = 1, rusanov = 2, ['euler-hllc'] = 3}
M.reconIndex = {['piecewise constant'] = 1, ['plm cons'] = 2, ['plm prim'] = 3, ['plm athena'] = 4}
M.precisionIndex = {['f64 plain'] = 0, f64 = 1, f32 = 2}
M.LAYOUT_AOS6_F64 = 0
M.initKind = {sod = 0, blast = 1, quadrant = 2, ['kelvin-helmholtz'] = 3}
M.ERR_BUDGET = -4
M.ERR_NO_SLOT = -5
M.renderMode = {heatmap = 0, volume = 1, lic = 2, slices = 3}

function M.check(code)
	if code ~= 0 then
		error('libhydrocuda: '..tostring(code)..': '..ffi.string(lib.hc_last_error()), 2)
	end
end

return M
