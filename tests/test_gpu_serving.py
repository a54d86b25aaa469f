"""Serving loop (fealpy_gb300.serving): requests arriving over time are
admitted into the running batch as slots and memory free up, every result
meets the 1e-10 true residual, matches the CPU oracle's solution of the same
request, and is the same (bit for bit) alone and in the mix."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return torch.device("cuda", 0)


def _stream():
    from fealpy_gb300.workloads import serving_requests
    # a short stream of small requests at a high arrival rate, so that many
    # arrive while others are still iterating; two of them elasticity solves
    reqs = serving_requests(24, rate=400.0, seed=11, dof_range=(3e2, 2e4))
    for k, n in ((5, 6), (13, 8)):
        reqs[k].update({"kind": "elast", "n": n, "p": 1, "dofs": 3 * (n + 1) ** 3})
    return reqs


def test_serving_mix_equals_solo_and_converges():
    dev = cuda()
    from fealpy_gb300.serving import SolveServer, poisson_request_problem
    from fealpy_gb300.batch import BatchSolver
    reqs = _stream()
    srv = SolveServer(max_slots=6, chunk=16, device=dev)
    out = srv.run(reqs, keep_solutions=True)
    assert out["n"] == len(reqs) and out["p99_s"] >= out["p50_s"] > 0
    assert out["max_relres"] <= 1e-10 * 1.0001
    assert srv.resident == 0 and srv.peak_resident > 0
    from oracle import fem_oracle as O
    for i, r in enumerate(reqs):
        inp = {}
        A, b = poisson_request_problem(r, dev, inputs=inp)
        bs = BatchSolver(1, max_slice_tiles=1 << 17, max_row_tiles=1 << 17, device=dev)
        bs.add(A, b, rtol=1e-10, maxit=100000, key=0)
        solo = bs.solve_all()[0]
        assert np.array_equal(solo.x.cpu().numpy(), out["solutions"][i]), i
        # against the CPU oracle's pipeline (reference algorithm) on the same inputs
        if inp["kind"] == "elast":
            ref = O.elasticity_pipeline(inp["node"], inp["cell"], 1.0 * inp["scale"], 0.5 * inp["scale"], q=4,
                                        clamp=lambda x: np.abs(x[..., 0]) < 1e-12, rtol=1e-12)
        else:
            ref = O.poisson_pipeline(inp["node"], inp["cell"], inp["p"], kappa=inp["kappa"], q=inp["p"] + 2,
                                     rtol=1e-12)
        err = np.max(np.abs(out["solutions"][i] - ref["x"])) / np.max(np.abs(ref["x"]))
        assert err < 1e-8, (i, inp["kind"], err)


def test_serving_memory_budget_limits_admission():
    dev = cuda()
    from fealpy_gb300.serving import SolveServer, resident_estimate
    reqs = _stream()[:8]
    # a budget of a little more than the largest request: one at a time
    big = max(resident_estimate(r["dofs"], 20 * r["dofs"], False) for r in reqs)
    srv = SolveServer(max_slots=8, chunk=16, hbm_budget=1.2 * big, device=dev)
    out = srv.run(reqs)
    assert out["n"] == len(reqs) and out["max_relres"] <= 1e-10 * 1.0001
    assert srv.peak_resident <= 1.2 * big


def test_serving_multigrid_lane_mix_equals_solo():
    """Requests above the lane threshold are solved by multigrid PCG beside the
    batch: every result meets 1e-10, a lane result equals the same request
    solved alone through the lane's path bit for bit, and matches the oracle."""
    dev = cuda()
    from fealpy_gb300.serving import SolveServer, poisson_request_problem, multigrid_solve
    from oracle import fem_oracle as O
    reqs = _stream()
    thr = sorted(r["dofs"] for r in reqs)[len(reqs) // 2]  # about half the requests in the lane
    srv = SolveServer(max_slots=6, chunk=16, device=dev, amg_min_dofs=thr)
    out = srv.run(reqs, keep_solutions=True)
    lane = [i for i, r in enumerate(reqs) if r["dofs"] >= thr]
    assert out["amg_lane_requests"] == len(lane) > 0
    assert out["max_relres"] <= 1e-10 * 1.0001
    for i in lane:
        assert out["info"][i]["lane"] == "amg" and out["info"][i]["niter"] < 200
        inp = {}
        A, b = poisson_request_problem(reqs[i], dev, inputs=inp)
        x, niter, _, relres = multigrid_solve(A, b, 1e-10, 100000)
        assert np.array_equal(x.cpu().numpy(), out["solutions"][i]), i
        assert niter == out["info"][i]["niter"] and relres == out["info"][i]["relres"]
        if inp["kind"] == "elast":
            ref = O.elasticity_pipeline(inp["node"], inp["cell"], 1.0 * inp["scale"], 0.5 * inp["scale"], q=4,
                                        clamp=lambda x: np.abs(x[..., 0]) < 1e-12, rtol=1e-12)
        else:
            ref = O.poisson_pipeline(inp["node"], inp["cell"], inp["p"], kappa=inp["kappa"], q=inp["p"] + 2,
                                     rtol=1e-12)
        err = np.max(np.abs(out["solutions"][i] - ref["x"])) / np.max(np.abs(ref["x"]))
        assert err < 1e-8, (i, inp["kind"], err)
