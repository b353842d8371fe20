"""The C-ABI library on a machine without a GPU: it builds, loads, exports
every entry point include/hydrocuda.h declares, and rejects bad arguments
before touching the device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "hydrocuda.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hc_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    import hydrocuda
    names = declared_functions()
    assert len(names) >= 30
    assert sorted(hydrocuda.PROTOTYPES) == names


def test_library_exports_every_declared_symbol():
    import hydrocuda
    L = hydrocuda.load_library()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert L.hc_version().decode() == "0.3"


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors of the ABI structs have the C compiler's sizes and field offsets."""
    import subprocess
    import hydrocuda
    structs = {"hc_solver_desc": hydrocuda.SolverDesc, "hc_batch_desc": hydrocuda.BatchDesc,
               "hc_done": hydrocuda.Done, "hc_batch_stats": hydrocuda.BatchStats, "hc_init": hydrocuda.Init,
               "hc_render": hydrocuda.Render}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "hydrocuda.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%%s %%zu\\n", "%s", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%%s.%%s %%zu\\n", "%s", "%s", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(l.split() for l in subprocess.check_output([str(exe)]).decode().splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got["%s.%s" % (cname, f)]) == getattr(py, f).offset, (cname, f)


def test_bad_arguments_fail_before_the_device():
    import hydrocuda
    L = hydrocuda.load_library()
    out = ctypes.c_void_p()
    d = hydrocuda.make_desc(dict(dim=2, gridSize=[8, 8]))
    assert L.hc_solver_create(None, ctypes.byref(d), ctypes.byref(out)) == -1
    assert L.hc_solver_status(None) == -1
    assert L.hc_batch_step(None, 1, None) == -1
    assert b"NULL" in L.hc_last_error()
    # the batched admission / fetch: a NULL batch or count array is refused
    got = ctypes.c_int(7)
    slots = (ctypes.c_int * 2)()
    assert L.hc_batch_admit_many(None, 2, ctypes.byref(d), None, 0, None, None, None, slots,
                                 ctypes.byref(got)) == -1
    assert L.hc_batch_admit_many(None, 0, None, None, 0, None, None, None, None, None) == -1
    assert L.hc_batch_fetch_many(None, 1, slots, None, 0) == -1
    assert b"NULL" in L.hc_last_error()


def test_descriptor_mapping_follows_reference_names():
    import hydrocuda
    d = hydrocuda.make_desc(dict(dim=3, gridSize=[4, 5, 6], boundary={"xmin": "mirror", "zmax": "periodic"},
                                 fluxLimiter="superbee", usePLM=None, integrator="Runge-Kutta 3, TVD",
                                 eqnArgs={"heatCapacityRatio": 5 / 3}))
    assert list(d.n) == [4, 5, 6]
    assert list(d.boundary) == [2, 3, 3, 3, 3, 1]
    assert d.flux_limiter == 18 and d.integrator == 9 and abs(d.gamma - 5 / 3) < 1e-15
    with pytest.raises(ValueError):
        hydrocuda.make_desc(dict(dim=1, gridSize=8, fluxLimiter="no such limiter"))
    assert hydrocuda.make_desc(dict(dim=1, gridSize=8, flux="hll")).flux == 1
    assert hydrocuda.make_desc(dict(dim=1, gridSize=8, flux="rusanov")).flux == 2
    with pytest.raises(ValueError):
        hydrocuda.make_desc(dict(dim=1, gridSize=8, flux="marquina"))
    assert hydrocuda.make_desc(dict(dim=1, gridSize=8, usePLM="plm prim")).recon == 3
    assert hydrocuda.make_desc(dict(dim=1, gridSize=8, usePLM="plm athena")).recon == 4
    with pytest.raises(ValueError):
        hydrocuda.make_desc(dict(dim=1, gridSize=8, usePLM="ppm"))


def test_render_defaults_without_a_device():
    """The reference's view defaults (integralMaxIter 10, 1024^2 noise, the
    identity slice rotation, palette 1) and rejection of unknown modes."""
    import hydrocuda
    r = hydrocuda.make_render("lic")
    assert (r.mode, r.lic_iter, r.noise_size, r.palette) == (2, 10, 1024, 0)
    assert list(r.slice_angle) == [0.0, 0.0, 0.0, 1.0]
    r = hydrocuda.make_render("heatmap", var="Mach number", palette="blue", width=64)
    assert (r.var, r.palette, r.width) == (hydrocuda.DISPLAY_VARS.index("Mach number"), 2, 64)
    L = hydrocuda.load_library()
    r = hydrocuda.make_render("slices")
    assert (r.num_slices, r.use_isobars, r.num_isobars, r.alpha) == (255, 1, 20.0, .15)
    assert L.hc_render_defaults(7, ctypes.byref(hydrocuda.Render())) == -1
    with pytest.raises(ValueError):
        hydrocuda.make_render("heatmap", var="vorticity")


def test_init_defaults_without_a_device():
    """hc_init_defaults is host-only: the reference's default states, no device needed."""
    import hydrocuda
    L = hydrocuda.load_library()
    ic = hydrocuda.Init()
    assert L.hc_init_defaults(0, ctypes.byref(ic)) == 0
    assert (ic.kind, list(ic.p[:4])) == (0, [1.0, 1.0, 0.125, 0.1])
    assert L.hc_init_defaults(3, ctypes.byref(ic)) == 0 and ic.seed == 2 and ic.p[0] == 0.01
    assert L.hc_init_defaults(7, ctypes.byref(ic)) == -1
    q = hydrocuda.make_init("quadrant", q=[(1, 2, 3, 4)] * 4)
    assert list(q.p) == [1, 2, 3, 4] * 4


def test_integration_c_example_compiles():
    """The C usage the integration notes show (tests/fixtures/integration_example.c)
    compiles against the header with every warning an error."""
    import subprocess
    src = os.path.join(ROOT, "tests", "fixtures", "integration_example.c")
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-Wno-unused-variable", "-fsyntax-only",
                           "-I", os.path.join(ROOT, "include"), src])


def test_noalloc_rejects_bad_descriptors_before_the_device():
    """hc_calc_dt_noalloc checks the fields it reads as solver creation does,
    and sizes before adding ghosts, without touching a device."""
    import hydrocuda
    L = hydrocuda.load_library()
    base = dict(dim=2, gridSize=[8, 8], mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow", cfl=.5)
    buf = ctypes.c_void_p(16)      # never dereferenced: every case fails first
    bad = []
    d = hydrocuda.make_desc(base); d.n[0] = 1; bad.append(d)                       # fewer than 2 cells
    d = hydrocuda.make_desc(base); d.maxs[1] = d.mins[1]; bad.append(d)           # empty extent
    d = hydrocuda.make_desc(base); d.gamma = 1.0; bad.append(d)                   # gamma not above 1
    d = hydrocuda.make_desc(base); d.cfl = 0.0; d.fixed_dt = 0.0; bad.append(d)   # no dt rule
    d = hydrocuda.make_desc(base); d.n[0] = 2 ** 31 - 2; bad.append(d)           # overflows with ghosts
    d = hydrocuda.make_desc(base); d.n[0] = 4096; d.n[1] = 4096; bad.append(d)    # beyond the scratch
    for d in bad:
        assert L.hc_calc_dt_noalloc(ctypes.byref(d), buf, buf, None) == -1
