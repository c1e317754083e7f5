"""SIRT: the reference recipe, the batched solver, and agreement between them."""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from oracle import oracle as orc
from tomosipo_gb300.sirt import BatchedSirt, sirt
from tests.helpers import ellipsoid_phantom, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


def _job(dev, n, cone, angles, seed):
    vg = ts.volume(shape=n, size=1)
    pg = (ts.cone(angles=angles, shape=(n, 3 * n // 2), size=np.sqrt(2), cone_angle=0.5) if cone
          else ts.parallel(angles=angles, shape=(n, 3 * n // 2), size=(1, 1.5)))
    A = ts.operator(vg, pg)
    x = torch.from_numpy(ellipsoid_phantom(vg.shape, n=8, seed=seed)).to(dev)
    y = A(x)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    y = y + 0.01 * float(y.max()) * torch.randn(y.shape, generator=gen).to(dev)
    return A, y, x


def test_sirt_converges(dev):
    A, y, x_true = _job(dev, 48, True, 72, seed=3)
    errs = []
    for n in (1, 5, 20):
        errs.append(rel_l2(sirt(A, y, n).cpu().numpy(), x_true.cpu().numpy()))
    assert errs[0] > errs[1] > errs[2]
    res = [float(torch.linalg.norm(y - A(sirt(A, y, n)))) for n in (1, 5, 20)]
    assert res[0] > res[1] > res[2]


def _oracle_sirt(vg, pg, y, iterations):
    """The same recipe with FP64 oracle operators (R, C clipped at 1 / 1e-8)."""
    with np.errstate(divide="ignore"):
        R = np.minimum(1 / orc.fp(vg, pg, np.ones(vg.shape)), 1e8)
        C = np.minimum(1 / orc.bp_matched(vg, pg, np.ones(y.shape)), 1e8)
    x = np.zeros(vg.shape)
    for _ in range(iterations):
        x += C * orc.bp_matched(vg, pg, R * (y - orc.fp(vg, pg, x)))
    return x


def test_sirt_matches_fp64_oracle(dev):
    """10 iterations on the GPU (fp32) vs the same recipe with FP64 oracle operators."""
    vg = ts.volume(shape=24, size=1)
    pg = ts.cone(angles=30, shape=(24, 36), size=np.sqrt(2), cone_angle=0.5)
    A = ts.operator(vg, pg)
    x_true = ellipsoid_phantom(vg.shape, n=5, seed=9).astype(np.float64)
    y = orc.fp(vg, pg, x_true)
    x_gpu = sirt(A, torch.from_numpy(y.astype(np.float32)).to(dev), 10).cpu().numpy()
    assert rel_l2(x_gpu, _oracle_sirt(vg, pg, y, 10)) <= 1e-5


def test_batched_equals_plain_and_alone_equals_mix(dev):
    jobs = [_job(dev, 32, False, 40, 1), _job(dev, 48, True, 60, 2), _job(dev, 40, True, 50, 3),
            _job(dev, 64, False, 90, 4)]
    n_it = 6
    plain = [sirt(A, y, n_it) for A, y, _ in jobs]
    mix = BatchedSirt([(A, y) for A, y, _ in jobs])
    mix.run(n_it, graph=False)
    for a, b in zip(mix.x, plain):
        assert torch.equal(a, b)
    alone = BatchedSirt([(jobs[1][0], jobs[1][1])])
    alone.run(n_it, graph=False)
    assert torch.equal(alone.x[0], mix.x[1])


def test_batched_graph_replay_equals_eager(dev):
    # more jobs than the batch's 8 streams, and 13 iterations as graphs of 5, 5 and 3
    jobs = [_job(dev, 16 + 4 * (i % 4), i % 2 == 0, 12 + 3 * i, 20 + i) for i in range(11)]
    eager = BatchedSirt([(A, y) for A, y, _ in jobs])
    eager.run(13, graph=False)
    graphed = BatchedSirt([(A, y) for A, y, _ in jobs])
    graphed.graph_iterations = 5
    graphed.run(13, graph=True)
    torch.cuda.synchronize()
    for (A, y, _), a, b in zip(jobs, eager.x, graphed.x):
        assert torch.equal(a, b)
    assert torch.equal(eager.x[3], sirt(jobs[3][0], jobs[3][1], 13))


def test_batched_multi_job_groups_equal_plain(dev):
    """More small jobs than one multi-job launch takes (two groups of one copy
    layout, one group of the other, a single job of a third kind) beside a job
    too large to join them; per-job iteration counts, some zero, so groups
    shrink between iterations. Every job equals the plain SIRT loop bit for bit."""
    from tomosipo_gb300.sirt import NativeBatch, SirtJobState

    jobs = []
    for i in range(53):
        n = (8, 12, 16, 20)[i % 4]
        A, y, _ = _job(dev, n, i % 3 != 0, 4 + (i * 7) % 13, 100 + i)
        if i >= 45:  # single-voxel copies: the other multi-job kernel
            A.projector.set_tuning(dev.index, fp_pair_layout=0)
        jobs.append((A, y))
    # a volume above 2^21 voxels keeps its own launches
    vg = ts.volume(shape=(130, 128, 128), size=(130 / 128, 1, 1))
    pg = ts.cone(angles=5, shape=(130, 192), size=(130 / 128 * np.sqrt(2), 1.5), cone_angle=0.5)
    A = ts.operator(vg, pg)
    jobs.append((A, A(torch.from_numpy(ellipsoid_phantom(vg.shape, n=4, seed=7)).to(dev))))
    counts = [(i * 5) % 4 for i in range(len(jobs))]
    states = [SirtJobState(A, y, None, dev) for A, y in jobs]
    nb = NativeBatch(states)
    nb.step_jobs(counts)
    torch.cuda.synchronize()
    for (A, y), st, k in zip(jobs, states, counts):
        assert torch.equal(st.x, sirt(A, y, k)), (A.domain_shape, k)
    nb.close()


def test_batched_tilted_detectors_equal_plain(dev):
    """Tilted detectors (the general backprojector), alone and beside a
    circular scan, on both matched backprojectors for the separable angles:
    the batch equals the plain SIRT loop bit for bit, and both are within the
    parity tolerance of the same recipe on the FP64 oracle's operators."""
    from oracle import oracle as orc

    vg = ts.volume(shape=16, size=1)
    R = ts.rotate(pos=0, axis=(1.0, 0.5, 0.2), angles=0.5)
    pg = R * ts.cone(angles=8, shape=(16, 24), size=1.5, src_orig_dist=3, src_det_dist=4).to_vec()
    # a helical scan whose detector tilts by a few degrees: separable and
    # general angles in one job
    t = np.linspace(0, 2 * np.pi, 12, endpoint=False)
    tilt = np.where(np.arange(12) % 3 == 0, 0.08, 0.0)
    src = np.stack([0.1 * t, -2.5 * np.cos(t), 2.5 * np.sin(t)], 1)
    det = np.stack([0.1 * t, 1.0 * np.cos(t), -1.0 * np.sin(t)], 1)
    dv = np.stack([np.cos(tilt), np.sin(tilt) * np.sin(t), np.sin(tilt) * np.cos(t)], 1) * 1.2 / 16
    du = np.stack([0 * t, np.sin(t), np.cos(t)], 1) * 1.6 / 24
    pg_mix = ts.cone_vec(shape=(16, 24), src_pos=src, det_pos=det, det_v=dv, det_u=du)
    for kernel in (0, 1):
        jobs = []
        for i, g in enumerate((pg, pg_mix)):
            A = ts.operator(vg, g)
            A.projector.set_tuning(dev.index, bp_kernel=kernel, bp_shape=0)
            x = torch.from_numpy(ellipsoid_phantom(vg.shape, n=4, seed=50 + i)).to(dev)
            jobs.append((A, A(x)))
        stats = jobs[1][0].projector.stats(dev.index)
        assert stats["general_bp_angles"] > 0 and stats["separable_bp_angles"] > 0
        A2, y2, _ = _job(dev, 24, True, 30, 51)
        b = BatchedSirt(jobs + [(A2, y2)])
        b.run(3, graph=False)
        for (A, y), xb in zip(jobs + [(A2, y2)], b.x):
            assert torch.equal(xb, sirt(A, y, 3)), kernel
        b.close()
    # the recipe itself against the oracle's on the mixed job (data from the oracle)
    y_np = orc.fp(vg, pg_mix, ellipsoid_phantom(vg.shape, n=4, seed=51).astype(np.float64))
    A = jobs[1][0]
    x_gpu = sirt(A, torch.from_numpy(y_np.astype(np.float32)).to(dev), 3).cpu().numpy()
    assert rel_l2(x_gpu, _oracle_sirt(vg, pg_mix, y_np, 3)) <= 1e-5


def test_batched_rejects_detector_supersampling(dev):
    vg = ts.volume(shape=16, size=1)
    A = ts.operator(vg, ts.cone(angles=8, shape=(16, 24), size=1.5, cone_angle=0.4),
                    detector_supersampling=2)
    with pytest.raises(RuntimeError, match="supersampling"):
        BatchedSirt([(A, torch.zeros(A.range_shape, device=dev))])


def test_server_results_same_alone_and_in_mix(dev):
    """Continuous batching: jobs arriving over time, different sizes; each result
    equals the same request run alone (and the plain SIRT loop)."""
    from tomosipo_gb300.serving import Request, SirtServer

    jobs = [_job(dev, 32, True, 40, 11), _job(dev, 48, True, 64, 12), _job(dev, 40, False, 50, 13)]
    reqs = [Request(i, A, y, iterations=4 + 2 * i, arrival=0.02 * i) for i, (A, y, _) in enumerate(jobs)]
    res = SirtServer(memory_budget=2 << 30).run(reqs)
    assert all(r.status == "done" for r in res)
    for r, (A, y, _) in zip(res, jobs):
        alone = SirtServer(memory_budget=2 << 30).run([Request(0, A, y, r_iters(reqs, r.id))])[0]
        assert torch.equal(r.x, alone.x)
        assert torch.equal(r.x, sirt(A, y, r_iters(reqs, r.id)))


def r_iters(reqs, rid):
    return next(q.iterations for q in reqs if q.id == rid)


def test_autotuned_batch_equals_plain(dev):
    """Autotuned forward schedules (one autotuner run per job shape) change the
    order of independent tiles only: the batch still equals the plain loop."""
    jobs = [_job(dev, 24, True, 30, 31), _job(dev, 24, True, 36, 32), _job(dev, 32, False, 20, 33)]
    b = BatchedSirt([(A, y) for A, y, _ in jobs], autotune=True)
    assert len(b.tuning) == 2  # two shapes: 24^3 cone (twice) and 32^3 parallel
    b.run(3, graph=False)
    for (A, y, _), xb in zip(jobs, b.x):
        assert torch.equal(xb, sirt(A, y, 3))
    b.close()
