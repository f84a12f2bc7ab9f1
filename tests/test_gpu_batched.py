"""Batched multi-scene launch: every scene of a batch advanced by one set of
launches must match the same scene on the CPU oracle, and a batch of many
small scenes must beat stepping them one by one."""
import numpy as np
import pytest
import torch

from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import scenarios as S
from reduced_mpm_stress_training_gb300.batched import BatchedMPM, autotune, time_chunk_size

from helpers import oracle_sim, rel, within_fp32_floor

pytestmark = pytest.mark.gpu


def _mixed_batch():
    scenes = [S.small_column(3000, 32, seed=1), S.small_column(5000, 48, material="metal", seed=2),
              S.small_column(1500, 24, seed=3, friction_angle=40.0),
              S.small_column(4000, 32, seed=4, E=5e5)]
    for s in scenes:
        s.dt = 1e-4
    return scenes


def test_each_scene_of_a_batch_matches_the_oracle(cuda):
    scenes = _mixed_batch()
    b = BatchedMPM(scenes, device=cuda, chunk_size=128)
    refs = [oracle_sim(s) for s in scenes]
    refs64 = [oracle_sim(s, bits=64) for s in scenes]
    for k in range(6):
        b.step(scenes[0].dt)
        for r, r64 in zip(refs, refs64):
            r.p2g2p(scenes[0].dt)
            r64.p2g2p(scenes[0].dt)
    torch.cuda.synchronize()
    assert b.engine.status() == 0
    for i, (r, r64) in enumerate(zip(refs, refs64)):
        n = scenes[i].n_particles
        x = b.export(A.FIELD_X, i).cpu().numpy()
        v = b.export(A.FIELD_V, i).cpu().numpy()
        F = b.export(A.FIELD_F, i).cpu().numpy()
        for name, g, a, a64 in (("x", x, r.x0 + r.u, r64.x0 + r64.u), ("F", F, r.F, r64.F)):
            tol = max(1e-5, 3.0 * rel(a, a64))
            assert rel(g, a.reshape(n, -1)) < tol, (i, name, rel(g, a.reshape(n, -1)), tol)
        # v carries the float32 SVD noise of the stress (stiff metal: mu = 3.8e6)
        ok, info = within_fp32_floor(v, r.v, r64.v)
        assert ok, (i, "v", info)


def test_autotuner_picks_a_candidate_and_caches(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("MPM_GB300_CACHE", str(tmp_path))
    scenes = _mixed_batch()
    c = autotune(scenes, device=cuda, candidates=(64, 128))
    assert c in (64, 128)
    assert (tmp_path / "autotune.json").exists()
    assert autotune(scenes, device=cuda, candidates=(64, 128)) == c  # cached


def test_batch_beats_one_by_one(cuda):
    scenes = [S.small_column(10000, 48, seed=10 + i) for i in range(16)]
    for s in scenes:
        s.dt = 1e-4
    batched = time_chunk_size(scenes, 128, cuda, steps=8)
    seq = sum(time_chunk_size([s], 128, cuda, steps=8) for s in scenes)
    print(f"batched {batched * 1e6:.1f} us/substep, one by one {seq * 1e6:.1f} us/substep")
    assert batched < seq
