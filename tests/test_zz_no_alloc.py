"""erlbm_batch_run_noalloc: the batched-run entry point for callers that cannot allocate GPU memory.

Such a caller (one whose own allocator owns the device, or whose loop may not pay for cudaMalloc and
the synchronisation of cudaFree) hands in device buffers it already owns; the library keeps its
scratch in a fixed static device array.  These tests call it through the C ABI with device buffers
made by the test, and check its results against erlbm_batch_run, which allocates its scratch per
call, on two calls in a row.  Kept in a file of its own, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def E():
    import erlbm_gb300 as m
    return m


def noalloc_fn():
    from erlbm_gb300 import _lib
    f = _lib.lib().erlbm_batch_run_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(_lib.BatchDesc), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return f


def run_noalloc(desc, specs, stream_torch):
    """Copies the run table to a device buffer, calls the entry point, returns the results."""
    import torch
    from erlbm_gb300 import _lib
    n = len(specs)
    arr = (_lib.RunSpec * n)(*specs)
    raw = np.frombuffer(bytes(arr), dtype=np.uint8)
    d_runs = torch.from_numpy(raw.copy()).to("cuda")
    d_out = torch.zeros(n * C.sizeof(_lib.BatchResult), dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(stream_torch):
        rc = noalloc_fn()(C.byref(desc), n, C.c_void_p(d_runs.data_ptr()), C.c_void_p(d_out.data_ptr()),
                          C.c_void_p(stream_torch.cuda_stream))
    assert rc == 0, _lib.lib().erlbm_last_error()
    stream_torch.synchronize()
    host = d_out.cpu().numpy().tobytes()
    res = (_lib.BatchResult * n).from_buffer_copy(host)
    return [(r.label, r.decided_step, r.steps_done, r.status, r.margin, r.energy) for r in res]


def same(a, b):
    """Equal result lists; a diverged run reports NaN energy in both, which must count as equal."""
    if len(a) != len(b):
        return False
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            if not (u == v or (isinstance(u, float) and isinstance(v, float) and np.isnan(u) and np.isnan(v))):
                return False
    return True


def as_tuples(results):
    return [(r["label"], r["decided_step"], r["steps_done"], r["status"], r["margin"], r["energy"]) for r in results]


def tg_runs(m, n):
    out = []
    for k in range(n):
        i, j = (37 * k) % 400, (91 * k + 13) % 400
        u0, tau, tnh = m.tg_map_params(i, j, 400, 400, m.OP_EXTREG if k % 2 else m.OP_REG, 0.65)
        out.append(dict(op=m.OP_EXTREG if k % 2 else m.OP_REG, tau=tau, tau_nh=tnh, u0=u0, n_steps=1500))
    return out


def ob_runs(m, n):
    out = []
    for k in range(n):
        u, tau, tnh = m.obstacle_map_params((53 * k) % 400, (29 * k + 7) % 400)
        out.append(dict(op=m.OP_EXTREG, tau=tau, tau_nh=tnh, u0=u, n_steps=1200))
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_allocating_entry_point_twice(precision):
    import torch
    from erlbm_gb300 import _lib
    m = E()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    # Taylor-Green map points (energy checks, tables built by the entry point)
    runs = tg_runs(m, 40)
    ref = as_tuples(m.batch_run(19, 16, 16, runs, precision=precision, energy_every=100, energy_factor=2.0,
                                init=m.INIT_TG_MAP))
    desc = _lib.BatchDesc(19, 16, 16, None, -1, -1, 1.0, 100, 2.0, 0, 10.0, m.INIT_TG_MAP, precision, 0)
    specs = [_lib.RunSpec(r["op"], r["tau"], r["tau_nh"], r["u0"], r["n_steps"], 0) for r in runs]
    for _ in range(2):
        assert same(run_noalloc(desc, specs, stream), ref)
    # obstacle channel (solid mask passed as a device pointer, boundary planes, density checks)
    nx, ny, solid = m.obstacle_geometry()
    runs = ob_runs(m, 24)
    ref = as_tuples(m.batch_run(19, nx, ny, runs, precision=precision, solid=solid, inlet_x=1, outlet_x=nx - 2,
                                density_check=True, density_limit=10.0, init=m.INIT_REST))
    d_solid = torch.from_numpy(solid.copy()).to("cuda")
    desc = _lib.BatchDesc(19, nx, ny, C.c_void_p(d_solid.data_ptr()), 1, nx - 2, 1.0, 0, 2.0, 1, 10.0,
                          m.INIT_REST, precision, 0)
    specs = [_lib.RunSpec(r["op"], r["tau"], r["tau_nh"], r["u0"], r["n_steps"], 0) for r in runs]
    for _ in range(2):
        assert same(run_noalloc(desc, specs, stream), ref)


def test_noalloc_rejects_what_it_cannot_hold():
    from erlbm_gb300 import _lib
    m = E()
    desc = _lib.BatchDesc(19, 16, 16, None, -1, -1, 1.0, 100, 2.0, 0, 10.0, m.INIT_TG_MAP, 0, 0)
    f = noalloc_fn()
    assert f(C.byref(desc), 16385, None, None, None) == -1
    assert b"16384" in _lib.lib().erlbm_last_error()
    desc.init = m.INIT_AOS
    assert f(C.byref(desc), 4, None, None, None) == -6
