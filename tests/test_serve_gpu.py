"""GPU test of the serving loop: a request's result is the same alone and in
the mix (requests overlapping on the device on separate streams), and the
mixed-precision result matches the FP64 one, within 1e-10 relative."""
import numpy as np
import pytest

from hephaestus_gb300 import serve as S

pytestmark = pytest.mark.gpu

TOL = 1e-10  # relative 2-norm difference of the final A of each request


def _stream():
    return S.make_stream(10, rate=300.0, seed=11, dof_range=(1e4, 1.5e5), steps=3)


def test_results_same_alone_and_in_the_mix():
    import torch

    free, _ = torch.cuda.mem_get_info()
    mix = S.GpuExecutor(slots=4, precision="mixed", rtol=1e-12, keep=True)
    done, wall = S.run_stream(_stream(), mix, budget_bytes=int(0.3 * free), slots=4)
    assert all(r.result["status"] == "OK" for r in done), [r.result for r in done]
    # overlap really happened: some request started before another finished
    spans = sorted((r.start, r.finish) for r in done)
    assert any(spans[k + 1][0] < spans[k][1] for k in range(len(spans) - 1))
    alone = S.GpuExecutor(slots=1, precision="mixed", rtol=1e-12, keep=True)
    ref64 = S.GpuExecutor(slots=1, precision="fp64", rtol=1e-12, keep=True)
    for r in _stream():
        alone(r, 0)
        ref64(r, 0)
    for rid, a_mix in mix.kept.items():
        a_alone = alone.kept[rid]
        a64 = ref64.kept[rid]
        nrm = np.linalg.norm(a64)
        assert nrm > 0
        assert np.linalg.norm(a_mix - a_alone) / nrm <= TOL, rid
        assert np.linalg.norm(a_mix - a64) / nrm <= TOL, rid
