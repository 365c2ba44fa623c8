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


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_refuses_bad_runs_alone(precision):
    """A bad run in the device-side table is refused on its own (status 8, not stepped); the valid
    BGK and MRT runs around it equal erlbm_batch_run's results for the same runs."""
    import torch
    from erlbm_gb300 import _lib
    m = E()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    good = []
    for k in range(12):
        u0, tau, _ = m.tg_map_params((41 * k) % 400, (67 * k + 5) % 400, 400, 400, m.OP_REG, 0.65)
        good.append(dict(op=m.OP_BGK if k % 2 else m.OP_MRT, tau=tau, tau_nh=0.65, u0=u0, n_steps=900))
    bad = [dict(op=m.OP_EXTREG, tau=0.0, tau_nh=0.65, u0=0.05, n_steps=100),      # tau <= 0
           dict(op=m.OP_EXTREG, tau=0.6, tau_nh=0.0, u0=0.05, n_steps=100),      # tau_nh = 0
           dict(op=7, tau=0.6, tau_nh=0.65, u0=0.05, n_steps=100),               # no such operator
           dict(op=m.OP_REG, tau=float("nan"), tau_nh=1.0, u0=0.05, n_steps=100),  # non-finite tau
           dict(op=m.OP_REG, tau=0.6, tau_nh=1.0, u0=0.05, n_steps=-3)]          # negative budget
    order = []  # interleave: a bad run after every third good one
    gi = bi = 0
    while gi < len(good) or bi < len(bad):
        for _ in range(3):
            if gi < len(good):
                order.append(("g", gi))
                gi += 1
        if bi < len(bad):
            order.append(("b", bi))
            bi += 1
    ref = as_tuples(m.batch_run(9, 16, 16, good, precision=precision, energy_every=100, energy_factor=2.0,
                                init=m.INIT_TG_MAP))
    desc = _lib.BatchDesc(9, 16, 16, None, -1, -1, 1.0, 100, 2.0, 0, 10.0, m.INIT_TG_MAP, precision, 0)
    runs = [good[i] if t == "g" else bad[i] for t, i in order]
    specs = [_lib.RunSpec(r["op"], r["tau"], r["tau_nh"], r["u0"], r["n_steps"], 0) for r in runs]
    for _ in range(2):
        got = run_noalloc(desc, specs, stream)
        for (t, i), res in zip(order, got):
            if t == "b":
                assert res[3] == 8 and res[0] == 0 and res[2] == 0, (i, res)
            else:
                assert res[3] & 8 == 0
                assert same([res], [ref[i]]), (i, res, ref[i])
    # MRT has no D3Q19 form: refused per run on a D3Q19 table
    desc19 = _lib.BatchDesc(19, 16, 16, None, -1, -1, 1.0, 100, 2.0, 0, 10.0, m.INIT_TG_MAP, precision, 0)
    spec = [_lib.RunSpec(m.OP_MRT, 0.6, 0.65, 0.05, 200, 0), _lib.RunSpec(m.OP_EXTREG, 0.6, 0.65, 0.05, 200, 0)]
    got = run_noalloc(desc19, spec, stream)
    assert got[0][3] == 8 and got[1][3] & 8 == 0 and got[1][2] == 200


def test_noalloc_full_table():
    """A call with ERLBM_NOALLOC_MAX_RUNS short runs uses the whole static table; it matches
    erlbm_batch_run on the same runs."""
    import torch
    from erlbm_gb300 import _lib
    m = E()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    n = 16384
    rng = np.random.default_rng(5)
    runs = []
    for k in range(n):
        u0, tau, tnh = m.tg_map_params(int(rng.integers(0, 400)), int(rng.integers(0, 400)), 400, 400,
                                       m.OP_EXTREG, 0.65)
        runs.append(dict(op=m.OP_EXTREG, tau=tau, tau_nh=tnh, u0=u0, n_steps=int(rng.integers(0, 120))))
    ref = as_tuples(m.batch_run(9, 8, 8, runs, precision=1, energy_every=100, energy_factor=2.0,
                                init=m.INIT_TG_MAP))
    desc = _lib.BatchDesc(9, 8, 8, None, -1, -1, 1.0, 100, 2.0, 0, 10.0, m.INIT_TG_MAP, 1, 0)
    specs = [_lib.RunSpec(r["op"], r["tau"], r["tau_nh"], r["u0"], r["n_steps"], 0) for r in runs]
    for _ in range(2):
        assert same(run_noalloc(desc, specs, stream), ref)


def test_noalloc_refuses_tg_tables_under_capture():
    """With ERLBM_INIT_TG_MAP the call copies tables from pageable host memory; on a stream under
    capture it returns ERLBM_E_UNSUPPORTED and leaves the capture intact."""
    import torch
    from erlbm_gb300 import _lib
    m = E()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    desc = _lib.BatchDesc(19, 16, 16, None, -1, -1, 1.0, 100, 2.0, 0, 10.0, m.INIT_TG_MAP, 1, 0)
    spec = [_lib.RunSpec(m.OP_EXTREG, 0.6, 0.65, 0.05, 100, 0)]
    run_noalloc(desc, spec, stream)  # the first call on the device, outside any capture
    arr = (_lib.RunSpec * 1)(*spec)
    d_runs = torch.from_numpy(np.frombuffer(bytes(arr), dtype=np.uint8).copy()).to("cuda")
    d_out = torch.zeros(C.sizeof(_lib.BatchResult), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        rc = noalloc_fn()(C.byref(desc), 1, C.c_void_p(d_runs.data_ptr()), C.c_void_p(d_out.data_ptr()),
                          C.c_void_p(stream.cuda_stream))
        d_out.add_(0)  # the capture still records work after the refusal
    assert rc == -6
    assert b"capture" in _lib.lib().erlbm_last_error()
