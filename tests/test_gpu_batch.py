"""Batched acquisitions (one persistent launch, CUDA-graph replay, autotuned
tile) against the same acquisitions run one by one."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small_jobs():
    import axonexa_gb300 as A
    from axonexa_gb300 import workloads as W
    jobs = W.batch_256(seed=11, n_sub=12, walker_scale=0.05, max_steps=600)
    return jobs


def _single(job, dev):
    import axonexa_gb300 as A
    if job.lattice is None:
        return A.run_single(job.basis[0], job.seqs, job.num_walkers, job.steps, job.timestep,
                            job.seed, device=dev)
    return A.run_lattice(job.lattice, job.basis, job.seqs, job.num_walkers, job.steps,
                         job.timestep, job.seed, relaxation=job.relaxation,
                         permeable=job.permeable, device=dev)


@pytest.mark.parametrize("tile,graph", [(256, True), (1024, False), (4096, True)])
def test_batch_matches_individual_runs(dev, tile, graph):
    import axonexa_gb300 as A
    jobs = _small_jobs()
    res = A.run_batch(jobs, tile=tile, use_graph=graph, device=dev)
    for j, (job, r) in enumerate(zip(jobs, res)):
        one = _single(job, dev)
        # identical trajectories; only the FP64 summation order differs
        np.testing.assert_allclose(r.mx, one.mx, rtol=0, atol=1e-9 * job.num_walkers, err_msg=str(j))
        np.testing.assert_allclose(r.my, one.my, rtol=0, atol=1e-9 * job.num_walkers, err_msg=str(j))
        assert r.walker_steps == one.walker_steps
        assert r.hits == one.hits


def test_batch_graph_replay_is_deterministic(dev):
    import axonexa_gb300 as A
    b_jobs = _small_jobs()
    b = A.Batch(b_jobs, tile=512, use_graph=True, device=dev)
    b.launch()
    r1 = b.read()
    b.launch()
    b.launch()
    r2 = b.read()
    for a, c in zip(r1, r2):
        np.testing.assert_array_equal(a.mx, c.mx)
        np.testing.assert_array_equal(a.my, c.my)
    info = b.info()
    # one persistent kernel per job class present (single cylinders, single
    # spheres, permeable and impermeable cylinder lattices) and the
    # partial-sum reduction
    classes = {(("lattice_perm" if j.permeable else "lattice") if j.lattice is not None
                else type(j.basis[0]).__name__) for j in b_jobs}
    assert info["items"] > 12 and info["kernel_launches"] == 1 + len(classes)
    b.close()


def test_autotuner_picks_a_valid_shape_and_caches_it(dev, tmp_path, monkeypatch):
    import axonexa_gb300 as A
    monkeypatch.setenv("AXX_AUTOTUNE_CACHE", str(tmp_path / "tune.tsv"))
    jobs = _small_jobs()
    best = A.autotune(jobs, probe_steps=100, device=dev)
    assert best["tile"] % 128 == 0 and best["tile"] >= 256
    assert best["blocks_per_sm"] >= 1 and best["ms"] > 0
    text = (tmp_path / "tune.tsv").read_text().split()
    assert str(best["tile"]) in text
    # tile 0 reads the cache
    b = A.Batch(jobs, tile=0, device=dev)
    assert b.info()["tile"] == best["tile"]
    b.close()
