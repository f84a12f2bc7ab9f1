"""CPU checks of the stress-decoder restatement (oracle/decoder.py) against the
PyTorch float32 restatement of the reference's NetDec
(offline_training_xhat_and_stress_and_mu/CROMnet_secondary.py:203-301), the
parameter packing, and the library's parameter count (no GPU)."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import decoder as OD
from reduced_mpm_stress_training_gb300 import _capi as A
from reduced_mpm_stress_training_gb300 import decoder as D

from helpers import netdec_torch


def _rows(n, label_dim, mu_dim, seed=0):
    rng = np.random.default_rng(seed)
    lab = rng.normal(0, 1, (n, label_dim))
    x = rng.uniform([0.35, 0.35, 0.05], [0.65, 0.65, 0.85], (n, 3))
    mu = rng.uniform(20, 40, (n, mu_dim))
    return np.concatenate([lab, x, mu], 1).astype(np.float32)


CASES = [dict(label_dim=6, scale_mlp=10, mu_dim=1, siren=False),
         dict(label_dim=6, scale_mlp=10, mu_dim=1, siren=True),
         dict(label_dim=4, scale_mlp=20, mu_dim=0, siren=False),
         dict(label_dim=0, scale_mlp=7, mu_dim=2, siren=False)]


def _stats(siren):
    if siren:
        return ((0.35, 0.35, 0.05), (0.65, 0.65, 0.85))
    return ((0.5, 0.5, 0.45), (0.09, 0.09, 0.23))


@pytest.mark.parametrize("case", CASES)
def test_numpy_restatement_matches_torch_float32(case):
    siren = case["siren"]
    sd = D.netdec_state_dict(**case, seed=3, x_stats=_stats(siren),
                             q_stats=((1.0, -2.0, 0.5, 3.0, 0.0, -1.0), (10.0, 20.0, 5.0, 10.0, 1.0, 2.0)))
    rows = _rows(2000, case["label_dim"], case["mu_dim"])
    blob = D.pack(sd, siren).numpy()
    hidden = 3 * case["scale_mlp"]
    q64 = OD.forward(blob, rows, case["label_dim"], case["mu_dim"], hidden, siren, 30.0)
    q32 = netdec_torch(sd, torch.from_numpy(rows), case["label_dim"], siren, 30.0).numpy()
    err = np.linalg.norm(q32 - q64) / np.linalg.norm(q64)
    assert err < (1e-5 if siren else 2e-6), err
    # the float32 path of the restatement lands as close as PyTorch's
    q_np32 = OD.forward(blob, rows, case["label_dim"], case["mu_dim"], hidden, siren, 30.0, dtype=np.float32)
    assert np.linalg.norm(q_np32 - q64) / np.linalg.norm(q64) < (1e-5 if siren else 2e-6)


def test_state_dict_prefix_and_symmetric_layout():
    sd = D.netdec_state_dict(seed=1)
    wrapped = {"decoder." + k: v for k, v in sd.items()}
    wrapped["encoder_unused.weight"] = torch.zeros(3)
    assert torch.equal(D.pack(wrapped, False), D.pack(sd, False))
    q = np.arange(12, dtype=np.float32).reshape(2, 6)
    S = OD.symmetric_stress(q).reshape(2, 3, 3)
    assert np.array_equal(S, np.swapaxes(S, 1, 2))
    assert np.array_equal(S[0][np.triu_indices(3)], q[0])   # [xx, xy, xz, yy, yz, zz]


def test_library_parameter_count(built):
    lib = A.load()
    for case in CASES:
        sd = D.netdec_state_dict(**case)
        d = A.MpmStressDecoder(0, case["label_dim"], case["mu_dim"], 3 * case["scale_mlp"], int(case["siren"]),
                               30.0, 0)
        assert lib.mpm_decoder_param_count(C.byref(d)) == D.pack(sd, case["siren"]).numel()
    bad = A.MpmStressDecoder(0, 6, 1, 65, 0, 30.0, 0)   # wider than the kernels take
    assert lib.mpm_decoder_param_count(C.byref(bad)) < 0


@pytest.mark.parametrize("siren", [False, True])
def test_decoder_golden(siren):
    """tests/golden/kat_decoder.json (hand-set weights, plain-math evaluation) against
    the packing + NumPy restatement and the PyTorch float32 restatement."""
    import json
    import os

    cases = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat_decoder.json")))
    g = next(c for c in cases if c["siren"] == siren)
    want = np.array(g["q"])
    # the packing and the restatement, in float64 on the fixture's exact values
    blob = D.pack(g["state_dict"], siren, dtype=torch.float64).numpy()
    q64 = OD.forward(blob, np.array(g["rows"]), g["label_dim"], g["mu_dim"], g["hidden"], siren, g["omega_0"])
    assert np.abs(q64 - want).max() <= 1e-9 * np.abs(want).max()
    if not siren:  # float32 weights and rows: ELU is well conditioned (sin(30 x) of inputs near 30 is not)
        sd = {k: torch.tensor(v, dtype=torch.float32) for k, v in g["state_dict"].items()}
        q32 = netdec_torch(sd, torch.tensor(g["rows"], dtype=torch.float32), g["label_dim"], siren,
                           g["omega_0"]).numpy()
        assert np.abs(q32 - want).max() <= 1e-5 * np.abs(want).max()
