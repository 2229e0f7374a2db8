"""Multi-session server (amcl_server_*): each session's results are identical to the
same filter stepped alone (whatever else is in flight, on one lane or spread over
concurrent lanes), admission refuses sessions
beyond the budget, and host-side failures (unknown session, a session that leaves
mid-stream, with requests still queued or running, NaN inputs) stay contained."""

import time

import numpy as np
import pytest

from amcl3d_gb300 import synth as S

pytestmark = pytest.mark.gpu

MODS = S.ODOM_MODS
ODOM = (*MODS, 0.05, 0.01, 0.0, 0.02)


@pytest.fixture(scope="module")
def scene(amcl):
    m = S.make_map(41, size_m=(10.0, 8.0, 3.0), n_boxes=10)
    G = amcl.Grid3d()
    G.buildGridMap(m.points, m.min, m.max, m.res, S.SENSOR_DEV)
    sessions = []
    for k, (P, n) in enumerate([(500, 300), (3000, 900), (12000, 600), (800, 0)]):
        pose = S.free_pose(m, 90 + k, height=1.2, clearance=0.4)
        scans = [S.ray_cast(m, pose, n_max=n, max_range=8.0, seed=5 * k + s) if n else np.zeros((0, 4), np.float32)
                 for s in range(3)]
        sessions.append(dict(P=P, pose=pose, scans=scans, ranges=S.beacons(m, pose, 3, seed=k), seed=500 + k))
    return G, sessions


def alone_means(amcl, G, sp, nreq):
    pf = amcl.ParticleFilter(seed=sp["seed"])
    x, y, z, a = sp["pose"]
    pf.init(sp["P"], x, y, z, a, 0.3, 0.3, 0.05, 0.1)
    out = []
    for r in range(nreq):
        pf.predict(*ODOM)
        pf.update(G, sp["scans"][r], sp["ranges"], 0.5, 0.1, 0.0, 0.0)
        m = pf.getMean()
        out.append(np.array([m.x, m.y, m.z, m.a], np.float32))
        pf.resample()
    return out


def drain(srv, n, timeout=60.0):
    got = []
    t0 = time.time()
    while len(got) < n and time.time() - t0 < timeout:
        got += srv.poll()
        time.sleep(0.001)
    return got


@pytest.mark.parametrize("lanes", [1, 4])
def test_sessions_match_alone_in_the_mix(amcl, scene, lanes):
    from amcl3d_gb300.serve import Server

    G, sessions = scene
    nreq = 3
    srv = Server(max_sessions=8, max_particles=40000, max_points_per_step=10000, lanes=lanes)
    sids = []
    for sp in sessions:
        x, y, z, a = sp["pose"]
        sid = srv.open_session(G, sp["P"], sp["seed"], sp["P"], [x, y, z, a, 0.3, 0.3, 0.05, 0.1])
        assert sid is not None
        sids.append(sid)
    # interleaved submissions: later requests arrive while earlier steps run
    tickets = {}
    for r in range(nreq):
        for sid, sp in zip(sids, sessions):
            tickets[srv.submit(sid, sp["scans"][r], sp["ranges"], ODOM)] = (sid, r)
    got = drain(srv, len(tickets))
    assert len(got) == len(tickets)
    per = {sid: {} for sid in sids}
    for ticket, sid, status, ts, td, mean in got:
        assert status == 0 and td >= ts
        per[sid][tickets[ticket][1]] = np.array(mean, np.float32)
    for sid, sp in zip(sids, sessions):
        want = alone_means(amcl, G, sp, nreq)
        for r in range(nreq):
            np.testing.assert_array_equal(per[sid][r], want[r], err_msg=f"session {sid} request {r}")
    st = srv.stats()
    assert st["requests"] == len(tickets) and st["steps"] >= nreq
    for sid in sids:
        srv.close_session(sid)
    srv.close()


def test_admission_and_host_failures(amcl, scene):
    from amcl3d_gb300 import _native as N
    from amcl3d_gb300.serve import Server

    G, sessions = scene
    srv = Server(max_sessions=2, max_particles=4000, max_points_per_step=4000)
    sp = sessions[1]
    x, y, z, a = sp["pose"]
    init = [x, y, z, a, 0.3, 0.3, 0.05, 0.1]
    s1 = srv.open_session(G, 3000, 1, 3000, init)
    assert s1 is not None
    assert srv.open_session(G, 3000, 2, 3000, init) is None  # budget exhausted: admission refused
    s2 = srv.open_session(G, 500, 3, 500, init)
    assert s2 is not None
    with pytest.raises(N.AmclError):
        srv.submit(987654, sp["scans"][0], sp["ranges"], ODOM)  # unknown session
    bad = sp["scans"][0].copy()
    bad[:10, 0] = np.nan  # NaN points are skipped by the weighting, as in the reference
    t_bad = srv.submit(s2, bad, sp["ranges"], ODOM)
    t_ok = srv.submit(s1, sp["scans"][0], sp["ranges"], ODOM)
    got = {r[0]: r for r in drain(srv, 2)}
    assert got[t_bad][2] == 0 and got[t_ok][2] == 0
    assert np.all(np.isfinite(got[t_ok][5]))
    # a session leaves between requests; its slot is reused by a new one
    srv.close_session(s1)
    s3 = srv.open_session(G, 3000, 4, 3000, init)
    assert s3 is not None
    t3 = srv.submit(s3, sp["scans"][1], sp["ranges"], ODOM)
    assert drain(srv, 1)[0][0] == t3
    srv.close()


@pytest.mark.parametrize("lanes", [1, 4])
def test_close_with_requests_queued(amcl, scene, lanes):
    """A session closed while its requests are still queued or on the GPU: the close
    waits for them (they complete, results delivered), frees the slot, and the other
    sessions' results are still exactly those of the same filters stepped alone."""
    from amcl3d_gb300.serve import Server

    G, sessions = scene
    nreq = 3
    srv = Server(max_sessions=8, max_particles=40000, max_points_per_step=10000, lanes=lanes)
    sids = []
    for sp in sessions:
        x, y, z, a = sp["pose"]
        sids.append(srv.open_session(G, sp["P"], sp["seed"], sp["P"], [x, y, z, a, 0.3, 0.3, 0.05, 0.1]))
    leaving = sids[2]  # the 12,000-particle session: its steps take longest
    tickets = {}
    for r in range(nreq):
        for sid, sp in zip(sids, sessions):
            tickets[srv.submit(sid, sp["scans"][r], sp["ranges"], ODOM)] = (sid, r)
    srv.close_session(leaving)  # returns once its queued and running requests are done
    got = drain(srv, len(tickets))
    assert len(got) == len(tickets)
    per = {sid: {} for sid in sids}
    for ticket, sid, status, ts, td, mean in got:
        assert status == 0
        per[sid][tickets[ticket][1]] = np.array(mean, np.float32)
    assert len(per[leaving]) == nreq
    for sid, sp in zip(sids, sessions):
        want = alone_means(amcl, G, sp, nreq)
        for r in range(nreq):
            np.testing.assert_array_equal(per[sid][r], want[r], err_msg=f"session {sid} request {r}")
    from amcl3d_gb300 import _native as N

    with pytest.raises(N.AmclError):
        srv.submit(leaving, sessions[2]["scans"][0], sessions[2]["ranges"], ODOM)  # gone
    x, y, z, a = sessions[2]["pose"]
    assert srv.open_session(G, 12000, 9, 12000, [x, y, z, a, 0.3, 0.3, 0.05, 0.1]) is not None  # slot reused
    for sid in sids:
        if sid != leaving:
            srv.close_session(sid)
    srv.close()
