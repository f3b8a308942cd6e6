"""The serving loop on the GPU: every request admitted under the budget runs
all its steps, and each result is the same as the request run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["lockstep", "free"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_served_results_equal_alone(precision, mode):
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
    if mode == "free":
        m = srv.run_free(stream, chunk=2, time_scale=1.0)
    else:
        m = srv.run(stream, time_scale=1.0)
    assert m["requests"] == 6 and m["rejected"] == 0
    assert srv.peak_used <= budget and 1 <= srv.peak_active <= 6
    for k, (t, wl, steps) in enumerate(stream):
        alone = serve._gpu_make_model(wl, precision)
        alone.run(steps, graph=False)
        torch.cuda.synchronize()
        assert np.array_equal(alone.var.state.cpu().numpy(), finals[k]), k


@pytest.mark.parametrize("mode", ["lockstep", "free"])
def test_a_failing_request_is_retired_alone(mode):
    """A request whose initial vorticity holds a NaN is retired after its
    first step with the reason; the requests beside it finish with the
    results they give alone; bogus requests are rejected at submission."""
    import torch
    from fluid2d_gb300 import serve, workloads as W
    stream = W.served_stream(count=4, rate=1000., seed=32, side_min=128, side_max=256,
                             steps_min=3, steps_max=5)
    t, wl, steps = stream[2]
    wl = dict(wl, fields={k: v.copy() for k, v in wl["fields"].items()})
    wl["fields"]["vorticity"][20, 20] = np.nan
    stream[2] = (t, wl, steps)
    stream.append((stream[-1][0], dict(stream[0][1], nx=2), 3))  # bogus grid
    finals = {}

    def keep(req):
        finals[req.rid] = req.model.var.state.cpu().numpy()

    srv = serve.Server(100e9, precision="fp64", nstreams=4, on_finish=keep)
    if mode == "free":
        m = srv.run_free(stream, chunk=1, time_scale=1.0)
    else:
        m = srv.run(stream, time_scale=1.0)
    assert m["requests"] == 3 and m["failed"] == 1 and m["rejected"] == 1
    assert srv.failed[0].rid == 2 and "non-finite" in srv.failed[0].error
    assert srv.failed[0].done == 1
    assert srv.rejected[0].rid == 4 and "grid" in srv.rejected[0].error
    for k in (0, 1, 3):
        t, w, st = stream[k]
        alone = serve._gpu_make_model(w, "fp64")
        alone.run(st, graph=False)
        torch.cuda.synchronize()
        assert np.array_equal(alone.var.state.cpu().numpy(), finals[k]), k
