"""The serving loop on the GPU: every request admitted under the budget runs
all its steps, and each result is the same as the request run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_served_results_equal_alone(precision):
    import torch
    from fluid2d_gb300 import serve, workloads as W
    stream = W.served_stream(count=6, rate=1000., seed=31, side_min=128, side_max=256,
                             steps_min=3, steps_max=6)
    # room for about two requests at a time: forces queueing and churn
    budget = 2 * max(serve.estimate_bytes(w, precision) for _, w, _ in stream)
    finals = {}

    def keep(req):
        finals[req.rid] = req.model.var.state.cpu().numpy()

    srv = serve.Server(budget, precision=precision, nstreams=4, on_finish=keep)
    m = srv.run(stream, time_scale=1.0)
    assert m["requests"] == 6 and m["rejected"] == 0
    assert max(n for _, n, _, _ in srv.ticks) <= 2 or srv.used <= budget
    for k, (t, wl, steps) in enumerate(stream):
        alone = serve._gpu_make_model(wl, precision)
        alone.run(steps, graph=False)
        torch.cuda.synchronize()
        assert np.array_equal(alone.var.state.cpu().numpy(), finals[k]), k
