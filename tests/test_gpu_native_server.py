"""The library's own serving loop (sph_server_*, worker thread in C++):
every job's result equals the job run alone, bit for bit, whatever else ran
beside it; queued and resident jobs can be cancelled; a job larger than the
capacity is refused at submit; wait() gives up after its timeout and can be
called again; several threads submit and wait at once; destroying a server
with jobs still pending returns."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def requests(seed, count, lo=900, hi=3000, kmin=3, kmax=8):
    from fluidsim import scenes, server
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        sc = scenes.request_scene(rng, lo=lo, hi=hi, kmin=kmin, kmax=kmax)
        out.append(server.Request(k, sc["params"], sc["pos"], sc["vel"], sc["dt"],
                                  sc["substeps"], sc["steps"], arrival=0.0))
    return out


def test_results_equal_alone_with_a_queue(gpu_lib):
    from fluidsim import server
    reqs = requests(91, 6)
    srv = server.NativeServer(2 * 3000 * server.bytes_per_particle(), 8, substeps=3)
    done, stats = srv.run(reqs, realtime=False)
    srv.close()
    assert stats["requests"] == len(reqs) and stats["batched_steps"] > 0
    assert stats["p99_step_ms"] >= stats["p50_step_ms"] > 0
    for r in reqs:
        for g, e in zip((done[r.rid].pos, done[r.rid].vel, done[r.rid].dens),
                        server.run_alone(r)):
            assert np.array_equal(g, e), r.rid


def test_cancel_refuse_and_timeout(gpu_lib):
    import fluidsim
    from fluidsim import server
    reqs = requests(92, 4, lo=2500, hi=2900, kmin=40, kmax=40)
    srv = server.NativeServer(2 * 2900 * server.bytes_per_particle(), 8, substeps=3)
    jobs = [srv.submit(r.params, r.pos, r.vel, r.dt, r.steps) for r in reqs]
    srv.cancel(jobs[3])                     # still queued (two fit at a time)
    srv.cancel(jobs[0])                     # resident or about to be
    for j in (jobs[0], jobs[3]):
        with pytest.raises(fluidsim.SphError) as e:
            srv.wait(j)
        assert e.value.code == -4
    with pytest.raises(fluidsim.SphError) as e:
        srv.wait(jobs[1], timeout=0.0)      # 40 steps are not done yet
    assert e.value.code == -4
    got = srv.wait(jobs[1])
    for g, w in zip(got, server.run_alone(reqs[1])):
        assert np.array_equal(g, w)
    srv.wait(jobs[2])
    big = np.zeros((10 * 2900, 3), np.float32)
    with pytest.raises(fluidsim.SphError) as e:
        srv.submit(reqs[0].params, big, None, reqs[0].dt, 1)
    assert e.value.code == -3
    st = srv.stats()
    assert st["cancelled"] == 2 and st["completed"] == 2
    assert st["status_flags"] == 0
    srv.close()


def test_concurrent_submitters(gpu_lib):
    from fluidsim import server
    reqs = requests(93, 8, lo=500, hi=1500)
    srv = server.NativeServer(4 * 1500 * server.bytes_per_particle(), 16, substeps=3)
    results, errors = {}, []

    def client(part):
        try:
            mine = [(r, srv.submit(r.params, r.pos, r.vel, r.dt, r.steps)) for r in part]
            for r, j in mine:
                results[r.rid] = srv.wait(j)
        except Exception as exc:  # surfaced below
            errors.append(exc)

    threads = [threading.Thread(target=client, args=(reqs[k::4],)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=120)
    srv.close()
    assert not errors and len(results) == len(reqs)
    for r in reqs:
        for g, e in zip(results[r.rid], server.run_alone(r)):
            assert np.array_equal(g, e), r.rid


def test_destroy_with_pending_jobs(gpu_lib):
    from fluidsim import server
    reqs = requests(94, 5, lo=2000, hi=3000, kmin=200, kmax=200)
    srv = server.NativeServer(2 * 3000 * server.bytes_per_particle(), 8, substeps=3)
    for r in reqs:
        srv.submit(r.params, r.pos, r.vel, r.dt, r.steps)
    srv.close()                             # returns while jobs are pending


def test_dispatcher_over_the_native_server(gpu_lib):
    """fluidsim.dispatch with the library's serving loop as the backend of
    each device (one GPU here): every result equals the request run alone."""
    from fluidsim import dispatch, server
    reqs = requests(95, 5)
    disp = dispatch.Dispatcher.native([0], 4 * 3000 * server.bytes_per_particle(),
                                      max_scenes=16, substeps=3)
    done, placed = disp.run(reqs)
    disp.close()
    assert set(placed.values()) == {0}
    for r in reqs:
        for g, w in zip(done[r.rid], server.run_alone(r)):
            assert np.array_equal(g, w)
