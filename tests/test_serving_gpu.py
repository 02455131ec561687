"""The continuous-batching server (csrc/serve.cu through CutServer): every
request's result is the same alone and in a mix of requests admitted at
different times, equals the plain solve of its inputs within the max-flow
tolerance, and memory is reused as requests retire."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
U_TOL = 1e-3


def _payload(seed, shape, sigma):
    from miccai2016_gb300.serving import helix_request
    return helix_request(shape, sigma, seed)


def _serve(payloads, reqs, stagger, num_iter=300, update=30, error_bound=1e-4, workspace_bytes=256 << 20):
    """reqs: (payload index, weighting, decay); stagger: steps between admissions."""
    import torch
    from miccai2016_gb300.serving import ATV_EIGS, CutServer
    srv = CutServer(num_iter=num_iter, update=update, error_bound=error_bound, workspace_bytes=workspace_bytes,
                    max_slots=16)
    out = {}
    queue = list(enumerate(reqs))
    budget = (num_iter // update + 2) * (len(reqs) + 1) * max(stagger, 1) + 1000   # bounded loop
    while queue or any("iterations" not in v for v in out.values()):
        budget -= 1
        assert budget > 0, "requests did not finish"
        if queue:
            tag, (pi, w, d) = queue[0]
            u = torch.empty(payloads[pi]["shape"], dtype=torch.float32).pin_memory()
            if srv.admit(tag, payloads[pi], w, d, ATV_EIGS, u):
                out[tag] = dict(u=u)
                queue.pop(0)
        for _ in range(stagger if queue else 1):
            srv.step()
        for tag, it, res in srv.poll():
            out[tag].update(iterations=it, residual=res)
    srv.close()
    return out


def _plain(p, w, d, num_iter=300, update=30, error_bound=1e-4):
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.continuous_cut_anisotropic_gpu import CmfCutQAnisotropicGpu
    from miccai2016_gb300.serving import ATV_EIGS
    prm = CmfCutQAnisotropicGpu.CutParameters()
    prm.num_iter, prm.update, prm.error_bound = num_iter, update, error_bound
    c = CmfCutQAnisotropicGpu(prm)
    alpha = P.nonterminal_weights(p["grad2"].numpy().astype(np.float64), w, d).astype(np.float32)
    u = c.execute(p["img"].numpy(), p["quats"].numpy(), ATV_EIGS, alpha, p["cs"].numpy(), p["ct"].numpy(),
                  verbose=False)
    return u, c.last_iterations


def _payloads():
    shapes = [((24, 40, 36), 0.6), ((48, 32, 40), 1.2), ((20, 64, 30), 0.3)]
    pls = []
    for k, (shape, sigma) in enumerate(shapes):
        p = _payload(10 + k, shape, sigma)
        p["shape"] = shape
        pls.append(p)
    return pls


REQS = [(0, 0.05, 30.0), (1, 0.02, 3.0), (2, 0.3, 100.0), (0, 0.5, 0.3), (1, 0.1, 1000.0), (2, 0.01, 10.0)]


def test_each_result_is_the_same_alone_and_in_the_mix():
    pls = _payloads()
    mix = _serve(pls, REQS, stagger=2)
    for tag, req in enumerate(REQS):
        alone = _serve(pls, [req], stagger=1)[0]
        assert mix[tag]["iterations"] == alone["iterations"]
        assert np.array_equal(mix[tag]["u"].numpy(), alone["u"].numpy()), tag


def test_served_results_match_plain_solves():
    pls = _payloads()
    mix = _serve(pls, REQS, stagger=3)
    for tag, (pi, w, d) in enumerate(REQS):
        u, it = _plain(pls[pi], w, d)
        assert abs(mix[tag]["iterations"] - it) <= 30
        if mix[tag]["iterations"] == it:
            assert np.max(np.abs(mix[tag]["u"].numpy() - u)) <= U_TOL, tag


def test_fixed_iterations_retire_at_num_iter():
    pls = _payloads()
    out = _serve(pls, REQS[:3], stagger=1, num_iter=90, error_bound=-1.0)
    for tag, (pi, w, d) in enumerate(REQS[:3]):
        assert out[tag]["iterations"] == 90
        u, it = _plain(pls[pi], w, d, num_iter=90, error_bound=-1.0)
        assert it == 90
        assert np.max(np.abs(out[tag]["u"].numpy() - u)) <= U_TOL


def test_admission_waits_for_memory_and_reuses_it():
    import torch
    from miccai2016_gb300.serving import ATV_EIGS, CutServer
    pls = _payloads()
    one = CutServer.request_bytes(pls[1]["shape"])
    from miccai2016_gb300 import _native as N
    tables = int(N.lib().m16_server_table_bytes(16, 1 << 21))
    srv = CutServer(num_iter=300, update=30, error_bound=1e-4, workspace_bytes=tables + 2 * one + (1 << 20),
                    max_slots=16)
    us = [torch.empty(pls[1]["shape"], dtype=torch.float32).pin_memory() for _ in range(3)]
    assert srv.admit(0, pls[1], 0.05, 30.0, ATV_EIGS, us[0])
    assert srv.admit(1, pls[1], 0.1, 10.0, ATV_EIGS, us[1])
    assert not srv.admit(2, pls[1], 0.2, 3.0, ATV_EIGS, us[2])   # no room for a third
    done = []
    for _ in range(2000):
        if len(done) == 2:
            break
        srv.step()
        done += srv.poll()
    assert len(done) == 2
    assert srv.admit(2, pls[1], 0.2, 3.0, ATV_EIGS, us[2])       # memory came back
    for _ in range(2000):
        if len(done) == 3:
            break
        srv.step()
        done += srv.poll()
    assert len(done) == 3
    info = srv.info()
    assert info["resident"] == 0 and info["draining"] == 0
    srv.close()
    u, it = _plain(pls[1], 0.2, 3.0)
    assert [t for t, _, _ in done][-1] == 2
    assert np.max(np.abs(us[2].numpy() - u)) <= U_TOL


def test_telemetry_counts_the_iterations_that_ran():
    """m16_server_info.voxel_iterations is the sum over the finished requests
    of voxels x iterations, and the steps' device time is positive."""
    import torch
    from miccai2016_gb300.serving import ATV_EIGS, CutServer
    pls = _payloads()
    srv = CutServer(num_iter=300, update=30, error_bound=1e-4, workspace_bytes=256 << 20, max_slots=16)
    info0 = srv.info()
    assert info0["voxel_iterations"] == 0 and info0["gpu_ms"] == 0.0
    reqs = [(0, 0.05, 30.0), (1, 0.2, 10.0), (2, 0.01, 100.0), (0, 0.5, 3.0)]
    done = {}
    for tag, (pi, w, d) in enumerate(reqs):
        u = torch.empty(pls[pi]["shape"], dtype=torch.float32, pin_memory=True)
        assert srv.admit(tag, pls[pi], w, d, ATV_EIGS, u)
    for _ in range(200):
        srv.step()
        for tag, it, res in srv.poll():
            done[tag] = it
        if len(done) == len(reqs):
            break
    assert len(done) == len(reqs)
    info = srv.info()
    want = sum(int(np.prod(pls[pi]["shape"])) * done[tag] for tag, (pi, _, _) in enumerate(reqs))
    assert info["voxel_iterations"] == want
    assert info["gpu_ms"] > 0.0
    srv.close()


def test_served_results_match_the_oracle():
    """Served requests (admitted at different times, fixed iteration count)
    against the CPU oracle directly, not only through the plain CUDA path."""
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.serving import ATV_EIGS
    from oracle import oracle as O
    pls = _payloads()
    reqs = REQS[:4]
    out = _serve(pls, reqs, stagger=2, num_iter=120, error_bound=-1.0)
    for tag, (pi, w, d) in enumerate(reqs):
        p = pls[pi]
        alpha = P.nonterminal_weights(p["grad2"].numpy().astype(np.float64), w, d).astype(np.float32)
        u, it, _ = O.maxflow_solve(p["img"].numpy(), p["quats"].numpy(), ATV_EIGS, alpha, p["cs"].numpy(),
                                   p["ct"].numpy(), num_iter=120, update=30, error_bound=-1.0)
        assert out[tag]["iterations"] == it == 120
        assert np.max(np.abs(out[tag]["u"].numpy() - u)) <= U_TOL, tag
