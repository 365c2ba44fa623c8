"""Request server: continuous batching, admission while others run, and results independent of the
mix (the same request alone and among others gives the same result, bit for bit)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def E():
    import erlbm_gb300 as m
    return m


def mix(m, rng, n):
    reqs = []
    for k in range(n):
        kind = [m.REQ_TG2D, m.REQ_TG_MAP_POINT, m.REQ_OBSTACLE, m.REQ_TG3D][k % 4]
        prec = [m.FP64, m.FP32_SHIFTED][(k // 4) % 2]
        steps = int(rng.integers(1, 300))
        if kind == m.REQ_TG2D:
            L = int(rng.choice([32, 64, 128]))
            u0 = 2.0 / L
            tau = 0.5 + 3 * u0 * L / 50.0
            reqs.append(dict(kind=kind, precision=prec, op=m.OP_EXTREG, L=L, tau=tau, tau_nh=0.65, u0=u0,
                             n_steps=steps))
        elif kind == m.REQ_TG_MAP_POINT:
            u0, tau, tnh = m.tg_map_params(int(rng.integers(0, 400)), int(rng.integers(0, 400)))
            reqs.append(dict(kind=kind, precision=prec, op=m.OP_EXTREG, tau=tau, tau_nh=tnh, u0=u0,
                             n_steps=steps * 10))
        elif kind == m.REQ_OBSTACLE:
            u, tau, tnh = m.obstacle_map_params(int(rng.integers(0, 400)), int(rng.integers(0, 400)))
            s = int(rng.integers(1, 3))
            reqs.append(dict(kind=kind, precision=prec, op=m.OP_EXTREG, sx=s, sy=s, tau=tau, tau_nh=tnh, u0=u,
                             n_steps=steps * 5))
        else:
            reqs.append(dict(kind=kind, precision=prec, op=m.OP_EXTREG, L=32, tau=0.55, tau_nh=0.65, u0=0.05,
                             n_steps=steps))
    return reqs


KEYS = ("status", "label", "steps_done", "decided_step", "energy", "margin", "lane")


def test_results_same_alone_and_in_mix():
    m = E()
    reqs = mix(m, np.random.default_rng(11), 24)
    with m.Server(hbm_budget_bytes=2 << 30) as srv:
        alone = []
        for r in reqs:
            alone.append(srv.wait(srv.submit(**r)))
        tickets = [srv.submit(**r) for r in reqs]
        together = [srv.wait(t) for t in tickets]
    for a, b, r in zip(alone, together, reqs):
        assert a["status"] == 0, (a, r)
        assert all(a[k] == b[k] or (np.isnan(a[k]) and np.isnan(b[k])) for k in KEYS), (a, b, r)


def test_continuous_admission():
    """Short requests submitted after a long one start and finish while the long one still runs."""
    m = E()
    with m.Server(hbm_budget_bytes=2 << 30) as srv:
        long_t = srv.submit(m.REQ_TG2D, m.FP64, L=512, tau=0.5 + 3 * (2 / 512) * 512 / 50, u0=2 / 512,
                            n_steps=3000)
        shorts = [srv.submit(m.REQ_TG_MAP_POINT, m.FP32_SHIFTED, tau=0.51, tau_nh=0.65, u0=0.1, n_steps=200)
                  for _ in range(50)]
        shorts += [srv.submit(m.REQ_TG2D, m.FP32_SHIFTED, L=64, tau=0.62, u0=2 / 64, n_steps=50) for _ in range(8)]
        rs = [srv.wait(t) for t in shorts]
        lr = srv.wait(long_t)
    assert all(r["status"] == 0 for r in rs)
    assert max(r["t_done"] for r in rs) < lr["t_done"]
    assert lr["steps_done"] == 3000


def test_server_results_match_oracle():
    m = E()
    with m.Server(hbm_budget_bytes=1 << 30) as srv:
        L, u0 = 32, 2 / 32
        tau = 0.5 + 3 * u0 * L / 50
        t = srv.submit(m.REQ_TG2D, m.FP64, op=m.OP_EXTREG, L=L, tau=tau, tau_nh=0.65, u0=u0, n_steps=77)
        r = srv.wait(t)
        lat = O.Lattice(9, L, L, 1, None, tau, 0.65, O.OP_EXTREG)
        lat.set(O.init_taylor_green(9, L, u0, tau))
        lat.step(77)
        assert r["energy"] == lat.kinetic_energy(0)
        # a map point through the resident loop equals the batched map kernel's result
        u0, tau, tnh = m.tg_map_params(300, 20)
        r = srv.wait(srv.submit(m.REQ_TG_MAP_POINT, m.FP64, tau=tau, tau_nh=tnh, u0=u0, n_steps=3623))
        lab, dec, mg = O.tg_map_point(16, O.OP_EXTREG, tau, tnh, u0)
        assert (r["label"], r["decided_step"], r["margin"]) == (lab, dec, mg)
        u, tau, tnh = m.obstacle_map_params(0, 0)
        r = srv.wait(srv.submit(m.REQ_OBSTACLE, m.FP64, sx=1, sy=1, tau=tau, tau_nh=tnh, u0=u, n_steps=2000))
        lab, dec, mg = O.obstacle_map_point(tau, tnh, u, max_steps=2000)
        assert (r["label"], r["decided_step"], r["margin"]) == (lab, dec, mg)
        r = srv.wait(srv.submit(m.REQ_OBSTACLE, m.FP64, sx=2, sy=2, tau=tau, tau_nh=tnh, u0=u, n_steps=500))
        lab, dec, mg = O.obstacle_map_point(tau, tnh, u, sx=2, sy=2, max_steps=500)
        assert (r["label"], r["decided_step"]) == (lab, dec)


def test_resident_loop_relaunches_after_idling_out():
    """The resident loop's CTAs leave after about half a second without work (a bounded wait); a
    request that arrives later relaunches it and gets the same result."""
    import time
    m = E()
    with m.Server(hbm_budget_bytes=1 << 28) as srv:
        u0, tau, tnh = m.tg_map_params(250, 40)
        a = srv.wait(srv.submit(m.REQ_TG_MAP_POINT, m.FP32_SHIFTED, tau=tau, tau_nh=tnh, u0=u0, n_steps=700))
        time.sleep(1.5)  # longer than the loop's idle limit
        b = srv.wait(srv.submit(m.REQ_TG_MAP_POINT, m.FP32_SHIFTED, tau=tau, tau_nh=tnh, u0=u0, n_steps=700),
                     timeout=60)
        for k in ("status", "label", "steps_done", "decided_step", "energy", "margin", "lane"):
            assert a[k] == b[k] or (a[k] != a[k] and b[k] != b[k]), k  # an unstable run reports NaN
        assert a["lane"] == 0


def test_wait_times_out_and_the_result_arrives_later():
    """erlbm_server_wait with a short limit returns ERLBM_E_TIMEOUT (-4) while the run is still going;
    the run finishes and a later wait returns it."""
    m = E()
    with m.Server(hbm_budget_bytes=1 << 30) as srv:
        t = srv.submit(m.REQ_TG3D, m.FP64, op=m.OP_EXTREG, L=64, tau=0.55, tau_nh=0.65, u0=0.05, n_steps=3000)
        with pytest.raises(m.ErlbmError) as ei:
            srv.wait(t, timeout=1e-3)
        assert ei.value.code == -4
        r = srv.wait(t, timeout=600)
        assert r["status"] == 0 and r["steps_done"] == 3000


def test_stream_lane_admits_the_shortest_runs_first():
    """With one stream the stream lane admits by estimated work (shortest first, aging with the
    wait), not by arrival: small lattices submitted after a large one start before it."""
    m = E()
    with m.Server(hbm_budget_bytes=1 << 30, max_streams=1, team_ctas=-1) as srv:
        blocker = srv.submit(m.REQ_TG2D, m.FP64, L=256, tau=0.6, tau_nh=0.65, u0=0.05, n_steps=3000)
        big = srv.submit(m.REQ_TG3D, m.FP64, op=m.OP_EXTREG, L=64, tau=0.55, tau_nh=0.65, u0=0.05, n_steps=2000)
        small = [srv.submit(m.REQ_TG2D, m.FP32_SHIFTED, L=128, tau=0.6, tau_nh=0.65, u0=0.05, n_steps=100)
                 for _ in range(4)]
        rb = srv.wait(big, timeout=600)
        rs = [srv.wait(t, timeout=600) for t in small]
        r0 = srv.wait(blocker, timeout=600)
        assert all(r["status"] == 0 for r in rs + [rb, r0])
        assert max(r["t_admit"] for r in rs) <= rb["t_admit"]
        assert r0["t_admit"] <= rb["t_admit"]


def test_large_2d_lattice_through_the_stream_lane():
    """A D2Q9 Taylor-Green side above 1024 (its initial-state table holds 4 L entries) is admitted and
    gives the oracle's energy; a side above 4096 is refused at submission.  The populations are the
    oracle's bit for bit (FP64), but the energy of 2.36 M nodes is a tree reduction on the device and a
    sequential sum in the oracle, so the two differ in the last digits (1.6e-14 relative measured)."""
    m = E()
    L, u0 = 1536, 2.0 / 1536
    tau = 0.5 + 3 * u0 * L / 50
    with m.Server(hbm_budget_bytes=1 << 30) as srv:
        r = srv.wait(srv.submit(m.REQ_TG2D, m.FP64, op=m.OP_EXTREG, L=L, tau=tau, tau_nh=0.65, u0=u0, n_steps=3),
                     timeout=600)
        with pytest.raises(m.ErlbmError) as ei:
            srv.submit(m.REQ_TG2D, m.FP64, L=4097, tau=tau, u0=u0, n_steps=3)
        assert ei.value.code == -1
    assert r["status"] == 0 and r["steps_done"] == 3 and r["lane"] == 1
    lat = O.Lattice(9, L, L, 1, None, tau, 0.65, O.OP_EXTREG)
    lat.set(O.init_taylor_green(9, L, u0, tau))
    lat.step(3)
    want = lat.kinetic_energy(0)
    assert abs(r["energy"] - want) <= 1e-12 * want


def tg3d_init(L, u0):
    """The server's 3-D Taylor-Green initial state restated on the host: rho = 1,
    u = u0 (sin kx cos ky cos kz, -cos kx sin ky cos kz, 0), dist_eq at every node (x fastest)."""
    x = np.arange(L, dtype=np.float64)
    s, c = np.sin(2. * np.pi * x / L), np.cos(2. * np.pi * x / L)
    f = np.empty((L, L, L, 19))
    for z in range(L):
        for y in range(L):
            for xx in range(L):
                ux = u0 * s[xx] * c[y] * c[z]
                uy = -u0 * c[xx] * s[y] * c[z]
                f[z, y, xx] = O.equilibrium(19, ux, uy, 0.0, 1.0)
    return f.reshape(-1)


@pytest.mark.parametrize("L,steps,exact", [(32, 40, True), (64, 6, False)])
def test_tg3d_requests_match_oracle(L, steps, exact):
    """Config-5 3-D Taylor-Green requests (D3Q19, L^3, FP64) through the server's resident team loop: the
    kinetic energy after the run equals the oracle's.  Up to 65536 nodes the device sums the energy
    serially in node order, as kinectic_energy does, so L = 32 matches bit for bit; L = 64 is a tree
    reduction, which agrees to the last digits only."""
    m = E()
    tau, tnh, u0 = 0.55, 0.65, 0.05
    with m.Server(hbm_budget_bytes=1 << 30) as srv:
        r = srv.wait(srv.submit(m.REQ_TG3D, m.FP64, op=m.OP_EXTREG, L=L, tau=tau, tau_nh=tnh, u0=u0, n_steps=steps),
                     timeout=600)
    assert r["status"] == 0 and r["steps_done"] == steps and r["lane"] == 2
    lat = O.Lattice(19, L, L, L, None, tau, tnh, O.OP_EXTREG)
    lat.set(tg3d_init(L, u0))
    lat.step(steps)
    want = lat.kinetic_energy(0)
    if exact:
        assert r["energy"] == want
    else:
        assert abs(r["energy"] - want) <= 1e-12 * want


@pytest.mark.parametrize("scale", [3, 4])
def test_scaled_obstacle_requests_match_oracle(scale):
    """Config-5 obstacle channels scaled 3x and 4x in each dimension (FP64, Zou-He inlet, density
    outlet, bounce-back, density checks every step): label, decided step and margin equal the oracle's
    roda_ponto on the same geometry, for a stable and an unstable point."""
    m = E()
    with m.Server(hbm_budget_bytes=1 << 30) as srv:
        for i, j, n in ((200, 399, 700), (10, 0, 700)):
            u, tau, tnh = m.obstacle_map_params(i, j)
            r = srv.wait(srv.submit(m.REQ_OBSTACLE, m.FP64, sx=scale, sy=scale, tau=tau, tau_nh=tnh, u0=u,
                                    n_steps=n), timeout=600)
            lab, dec, mg = O.obstacle_map_point(tau, tnh, u, sx=scale, sy=scale, max_steps=n)
            assert r["status"] == 0
            assert (r["label"], r["decided_step"], r["margin"]) == (lab, dec, mg), (i, j, r, lab, dec, mg)


def team_requests(m):
    """Requests of the resident team loop: D2Q9 Taylor-Green (energy summed serially up to 65536
    nodes, as a tree above), D3Q19 Taylor-Green, obstacle channels scaled 2x and 3x with a stable and
    an unstable point (density checks every step), in both precisions."""
    reqs = []
    for prec in (m.FP64, m.FP32_SHIFTED):
        for L, steps in ((64, 120), (256, 40), (512, 6)):
            u0 = 2.0 / L
            reqs.append(dict(kind=m.REQ_TG2D, precision=prec, op=m.OP_EXTREG, L=L, tau=0.5 + 3 * u0 * L / 50.0,
                             tau_nh=0.65, u0=u0, n_steps=steps))
        reqs.append(dict(kind=m.REQ_TG3D, precision=prec, op=m.OP_REG, L=32, tau=0.55, tau_nh=1.0, u0=0.05,
                         n_steps=30))
        for (i, j), s in (((200, 399), 2), ((10, 0), 3)):
            u, tau, tnh = m.obstacle_map_params(i, j)
            reqs.append(dict(kind=m.REQ_OBSTACLE, precision=prec, op=m.OP_EXTREG, sx=s, sy=s, tau=tau, tau_nh=tnh,
                             u0=u, n_steps=600))
    reqs.append(dict(kind=m.REQ_TG2D, precision=m.FP64, op=m.OP_MRT, L=128, tau=0.6, tau_nh=0.65, u0=0.02,
                     n_steps=50))
    return reqs


RESULT_KEYS = ("status", "label", "steps_done", "decided_step", "energy", "margin")


def same(a, b):
    return all(a[k] == b[k] or (np.isnan(a[k]) and np.isnan(b[k])) for k in RESULT_KEYS)


def test_team_loop_results_equal_the_stream_lane():
    """The resident team loop gives the stream lane's results bit for bit (the same per-node update,
    density fold and energy reduction shape): each request alone on a server without team loop
    (team_ctas < 0, lane 1) and on one whose team loop takes lattices up to 2^19 nodes (lane 2)."""
    m = E()
    reqs = team_requests(m)
    with m.Server(hbm_budget_bytes=1 << 30, team_ctas=-1) as srv:
        want = [srv.wait(srv.submit(**r), timeout=600) for r in reqs]
    with m.Server(hbm_budget_bytes=1 << 30, team_max_nodes=1 << 19) as srv:
        got = [srv.wait(srv.submit(**r), timeout=600) for r in reqs]
    assert all(w["lane"] == 1 for w in want) and all(g["lane"] == 2 for g in got)
    for r, w, g in zip(reqs, want, got):
        assert w["status"] == 0, (r, w)
        assert same(w, g), (r, w, g)
    assert any(g["label"] == 1 for g in got) and any(g["label"] == 0 and g["margin"] > 0 for g in got)


def test_team_loop_results_do_not_depend_on_the_team_size_or_the_mix():
    """The same requests one at a time on a team loop of three worker CTAs (team_ctas = 4), and all at
    once on the default loop, where each run is worked on by as many CTAs as join it: equal results,
    bit for bit."""
    m = E()
    reqs = team_requests(m)
    with m.Server(hbm_budget_bytes=1 << 30, team_ctas=4, team_max_nodes=1 << 19) as srv:
        small = [srv.wait(srv.submit(**r), timeout=600) for r in reqs]
    with m.Server(hbm_budget_bytes=1 << 30, team_max_nodes=1 << 19) as srv:
        tickets = [srv.submit(**r) for r in reqs]
        mixed = [srv.wait(t, timeout=600) for t in tickets]
    for r, a, b in zip(reqs, small, mixed):
        assert a["status"] == 0 and a["lane"] == 2 and b["lane"] == 2, (r, a)
        assert same(a, b), (r, a, b)


def test_team_loop_admits_by_footprint():
    """With a budget whose team pages hold one 512^2 FP64 lattice at a time (38 MB of populations in a
    64 MB team region), three of them run one after the other, while small requests are admitted
    beside them; every run completes with the result it has alone."""
    m = E()
    L = 512
    u0 = 2.0 / L
    big = dict(kind=m.REQ_TG2D, precision=m.FP64, op=m.OP_EXTREG, L=L, tau=0.5 + 3 * u0 * L / 50.0, tau_nh=0.65,
               u0=u0, n_steps=20)
    small = dict(kind=m.REQ_TG2D, precision=m.FP64, op=m.OP_EXTREG, L=64, tau=0.56, tau_nh=0.65, u0=2 / 64,
                 n_steps=200)
    with m.Server(hbm_budget_bytes=128 << 20, team_max_nodes=1 << 19) as srv:
        alone_big = srv.wait(srv.submit(**big), timeout=600)
        alone_small = srv.wait(srv.submit(**small), timeout=600)
        tb = [srv.submit(**big) for _ in range(3)]
        ts = [srv.submit(**small) for _ in range(6)]
        rb = [srv.wait(t, timeout=600) for t in tb]
        rs = [srv.wait(t, timeout=600) for t in ts]
    assert alone_big["lane"] == 2 and alone_small["lane"] == 2
    assert all(same(r, alone_big) for r in rb) and all(same(r, alone_small) for r in rs)
    run = alone_big["t_done"] - alone_big["t_admit"]
    admits = sorted(r["t_admit"] for r in rb)
    assert admits[1] - admits[0] > 0.3 * run and admits[2] - admits[1] > 0.3 * run  # one big run at a time
    assert max(r["t_admit"] for r in rs) < admits[2]  # the small runs did not wait behind the big ones


def test_team_loop_reports_a_phase_wait_that_runs_out():
    """A team-loop run whose phase waits are limited to 1 us (team_wait_us) cannot wait for its steps'
    previous phases: the wait runs out, the run goes on without it and ends with ERLBM_E_TIMEOUT
    (-4).  A run on a server with the default limit gives the result it has alone."""
    m = E()
    req = dict(kind=m.REQ_TG2D, precision=m.FP64, op=m.OP_EXTREG, L=256, tau=0.6, tau_nh=0.65, u0=0.02,
               n_steps=200)
    with m.Server(hbm_budget_bytes=1 << 30, team_wait_us=1) as srv:
        r = srv.wait(srv.submit(**req), timeout=600)
    assert r["lane"] == 2 and r["status"] == -4, r
    with m.Server(hbm_budget_bytes=1 << 30) as srv:
        ok = srv.wait(srv.submit(**req), timeout=600)
    assert ok["lane"] == 2 and ok["status"] == 0 and ok["steps_done"] == 200
