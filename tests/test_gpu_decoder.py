"""GPU parity of the reference's stress decoder (NetDec,
offline_training_xhat_and_stress_and_mu/CROMnet_secondary.py:203-301) run by
the library (mpm_decoder_forward, mpm_decoder_stress), against the float64
NumPy restatement (oracle/decoder.py) and the PyTorch float32 restatement.

Tolerance: 1e-5 relative L2 against the float64 restatement (PyTorch float32
itself lands at 3e-7 with ELU and 1.2e-6 with sin(30 x)); the decoded stress
in the particle state bit-matches the symmetric expansion of the GPU's own
row decode up to the order of the label's sum (1e-6)."""
import numpy as np
import pytest
import torch

from oracle import decoder as OD
from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import decoder as D
from reduced_mpm_stress_training_gb300 import scenarios as S

from helpers import gpu_sim, gpu_state, netdec_torch, rel

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _rows(n, label_dim, mu_dim, seed=0):
    rng = np.random.default_rng(seed)
    lab = rng.normal(0, 1, (n, label_dim))
    x = rng.uniform([0.35, 0.35, 0.05], [0.65, 0.65, 0.85], (n, 3))
    mu = rng.uniform(20, 40, (n, mu_dim))
    return np.concatenate([lab, x, mu], 1).astype(np.float32)


def _stats(siren):
    if siren:
        return ((0.35, 0.35, 0.05), (0.65, 0.65, 0.85))
    return ((0.5, 0.5, 0.45), (0.09, 0.09, 0.23))


Q_STATS = ((100.0, -20.0, 5.0, 300.0, 0.0, -100.0), (1e3, 2e2, 5e1, 1e3, 1e1, 2e3))


@pytest.mark.parametrize("case", [dict(label_dim=6, scale_mlp=10, mu_dim=1, siren=False),
                                  dict(label_dim=6, scale_mlp=10, mu_dim=1, siren=True),
                                  dict(label_dim=6, scale_mlp=20, mu_dim=1, siren=False),
                                  dict(label_dim=16, scale_mlp=21, mu_dim=0, siren=True),
                                  dict(label_dim=0, scale_mlp=3, mu_dim=2, siren=False)])
def test_decoder_forward_matches_restatements(cuda, case):
    siren = case["siren"]
    dec = D.StressDecoder.random(**case, seed=5, x_stats=_stats(siren), q_stats=Q_STATS, device=cuda)
    rows = _rows(50_000, case["label_dim"], case["mu_dim"])
    got = dec.forward(torch.from_numpy(rows)).cpu().numpy()
    q64 = OD.forward(dec.params.cpu().numpy(), rows, case["label_dim"], case["mu_dim"], dec.hidden, siren, 30.0)
    q32 = netdec_torch(dec.state_dict, torch.from_numpy(rows), case["label_dim"], siren, 30.0).numpy()
    assert rel(got, q64) <= TOL, (rel(got, q64), rel(q32, q64))
    assert rel(got, q32) <= TOL
    assert dec.forward(torch.empty((0, dec.n_in))).shape == (0, 6)


def test_decoded_stress_feeds_the_substep(cuda):
    """The loop the reference's reduced-order model runs: decode every particle's
    stress from (label, x_initial, friction angle), then a substep; against the
    same substep after load_uvstress_from_tensor of the row decode."""
    sc = S.small_column(8192, 32)
    n = sc.n_particles
    dec = D.StressDecoder.random(seed=2, x_stats=_stats(False), q_stats=Q_STATS, device=cuda)
    label = torch.from_numpy(np.random.default_rng(4).normal(0, 1, 6).astype(np.float32))
    a, b = gpu_sim(sc), gpu_sim(sc)
    for s in (a, b):
        s.p2g2p(0, sc.dt)
    a.load_stress_from_decoder(dec, label)
    x0, _, _, _ = sc.particles()
    rows = np.concatenate([np.tile(label.numpy(), (n, 1)), x0, np.full((n, 1), sc.friction_angle, np.float32)], 1)
    q = dec.forward(torch.from_numpy(rows)).cpu().numpy()
    q64 = OD.forward(dec.params.cpu().numpy(), rows, 6, 1, dec.hidden, False, 30.0)
    stress_a = a.mpm_state.particle_stress.cpu().numpy().reshape(n, 9)
    assert rel(stress_a, OD.symmetric_stress(q64)) <= TOL
    # the stress form runs the hidden layers on the tensor cores (three-piece
    # BF16 split), the row form on the CUDA cores in FP32: both land within
    # about 3e-7 of float64
    assert rel(stress_a, OD.symmetric_stress(q)) <= 2e-6
    u, v, _, _ = b.export_uvFstress_from_warp()
    b.load_uvstress_from_tensor(u, v, torch.from_numpy(OD.symmetric_stress(q)))
    for s in (a, b):
        s.p2g2p(1, sc.dt)
        s.check_status()
    ga, gb = gpu_state(a), gpu_state(b)
    for f in ("x", "v", "C", "F", "stress"):
        assert rel(ga[f], gb[f]) <= TOL, f


@pytest.mark.parametrize("case", [dict(label_dim=6, scale_mlp=10, mu_dim=1, siren=False),
                                  dict(label_dim=6, scale_mlp=10, mu_dim=1, siren=True),
                                  dict(label_dim=0, scale_mlp=3, mu_dim=2, siren=False),
                                  dict(label_dim=16, scale_mlp=2, mu_dim=0, siren=True),
                                  dict(label_dim=64, scale_mlp=10, mu_dim=4, siren=False),
                                  dict(label_dim=6, scale_mlp=20, mu_dim=1, siren=False)])
def test_decoded_stress_matches_float64_for_each_width(cuda, case):
    """mpm_decoder_stress against the float64 restatement on (label, x_initial,
    mu by uid) rows: widths up to 32 take the tensor-core kernel (128-particle
    tiles; 5,003 particles leave a ragged last tile), wider ones the CUDA-core
    kernel.  Same 1e-5 bar as the row form."""
    siren = case["siren"]
    sc = S.small_column(5003, 32)
    n = sc.n_particles
    sim = gpu_sim(sc)
    dec = D.StressDecoder.random(**case, seed=7, x_stats=_stats(siren), q_stats=Q_STATS, device=cuda)
    rng = np.random.default_rng(11)
    label = rng.normal(0, 1, case["label_dim"]).astype(np.float32)
    mu = rng.uniform(20, 40, (n, case["mu_dim"])).astype(np.float32)
    sim.load_stress_from_decoder(dec, torch.from_numpy(label), torch.from_numpy(mu) if case["mu_dim"] else None)
    assert sim.check_status() == 0
    x0, _, _, _ = sc.particles()
    rows = np.concatenate([np.tile(label, (n, 1)), x0, mu], 1).astype(np.float32)
    q64 = OD.forward(dec.params.cpu().numpy(), rows, case["label_dim"], case["mu_dim"], dec.hidden, siren, 30.0)
    got = sim.mpm_state.particle_stress.cpu().numpy().reshape(n, 9)
    assert rel(got, OD.symmetric_stress(q64)) <= TOL, (dec.hidden, rel(got, OD.symmetric_stress(q64)))


@pytest.mark.parametrize("n", [1, 100, 129])
def test_decoded_stress_with_fewer_particles_than_two_tiles(cuda, n):
    """The tensor-core stress decoder with one CTA whose second tile pipeline
    has no tile (n <= 128) or only a 1-row tile (n = 129): every particle's
    stress still matches float64."""
    sc = S.small_column(n, 16)
    sim = gpu_sim(sc)
    dec = D.StressDecoder.random(seed=9, x_stats=_stats(False), q_stats=Q_STATS, device=cuda)
    label = np.random.default_rng(3).normal(0, 1, 6).astype(np.float32)
    sim.load_stress_from_decoder(dec, torch.from_numpy(label))
    assert sim.check_status() == 0
    x0, _, _, _ = sc.particles()
    rows = np.concatenate([np.tile(label, (n, 1)), x0, np.full((n, 1), sc.friction_angle, np.float32)], 1)
    q64 = OD.forward(dec.params.cpu().numpy(), rows, 6, 1, dec.hidden, False, 30.0)
    got = sim.mpm_state.particle_stress.cpu().numpy().reshape(n, 9)
    assert rel(got, OD.symmetric_stress(q64)) <= TOL


def test_decoder_arguments_are_checked(cuda):
    sc = S.small_column(1024, 16)
    sim = gpu_sim(sc)
    dec = D.StressDecoder.random(device=cuda)
    with pytest.raises(ValueError):
        dec.stress_into(sim.engine, torch.zeros(5), torch.zeros(1024, 1))
    with pytest.raises(ValueError):
        dec.forward(torch.zeros(4, dec.n_in + 1))
    import ctypes as C

    lib = A.load()
    bad = A.MpmStressDecoder(dec.params.data_ptr(), 6, 1, 65, 0, 30.0, 0)
    assert lib.mpm_decoder_forward(C.byref(bad), 0, 0, 0, 0) == A.MPM_ERR_ARG
