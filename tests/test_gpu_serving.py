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
