"""The continuous-batching loop on the GPU: jobs of different types and
sizes overlap on the device, and each job's result is the same alone and in
the mix (within the mixed form's tolerance, 1e-5 relative on sigma)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from pyloworder_gb300 import serving  # noqa: E402


def _close(a, b, key):
    a, b = np.asarray(a), np.asarray(b)
    k = min(len(a), len(b), 6)
    if key == "mu":
        for z in a[:k]:
            assert np.min(np.abs(b - z)) < 1e-4
        return
    np.testing.assert_allclose(a[:k], b[:k], rtol=1e-5, atol=1e-7 * np.abs(b).max())


def test_same_result_alone_and_in_mix():
    jobs = serving.make_mix(10, seed=7, m_range=(16384, 131072), n_range=(32, 160))
    srv = serving.Server(hbm_budget_bytes=20e9, slots=4)
    done, summ = srv.run(jobs, realtime=False)
    assert summ["completed"] == len(jobs), [j.error for j in done if j.error]
    by = {j.jid: j for j in done}
    for jid in (0, 3, 6, 9):
        alone = serving.Job(jid, by[jid].kind, by[jid].m, by[jid].n, by[jid].seed)
        res = serving.Server(hbm_budget_bytes=20e9, slots=1).run([alone], realtime=False)[0][0]
        assert not res.error, res.error
        for key in res.result:
            if key in ("f",):
                continue
            _close(by[jid].result[key], res.result[key], key)


def test_jobs_on_different_streams_overlap_on_the_device():
    """Two admitted jobs run on their own streams at the same time: the
    device-side intervals between the events each job records on its stream
    intersect (the second starts before the first ends), and the two streams
    are different."""
    jobs = [serving.Job(0, "POD", 262144, 256, seed=1), serving.Job(1, "DMD", 262144, 200, seed=2),
            serving.Job(2, "POD", 131072, 300, seed=3), serving.Job(3, "SPOD", 131072, 400, seed=4)]
    srv = serving.Server(hbm_budget_bytes=40e9, slots=4)
    warm = serving.Server(hbm_budget_bytes=40e9, slots=4)
    warm.run([serving.Job(9, k, 65536, 96, seed=9) for k in ("POD", "DMD", "SPOD")], realtime=False)
    ref = torch.cuda.Event(enable_timing=True)
    ref.record()
    done, summ = srv.run(jobs, realtime=False)
    assert summ["completed"] == 4, [j.error for j in done if j.error]
    tl = srv.timeline(ref)
    assert len(tl) == 4 and len({w for _, w, _, _ in tl}) >= 2
    overlaps = [(a, b) for a in tl for b in tl
                if a[0] < b[0] and a[1] != b[1] and a[2] < b[3] and b[2] < a[3]]
    assert overlaps, tl
