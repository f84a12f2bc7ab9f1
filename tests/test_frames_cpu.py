"""Host logic of the frame files (save_data_at_frame / load_from_sampling /
load_uvFstress_from_h5, engine_stress/mpm_solver_warp.py:129-153, 268-404):
names, the device buffer's layout, the six stress components, OBJ text, and
the NumPy fallback store used where h5py is not importable (no GPU)."""
import os

import numpy as np
import pytest

from reduced_mpm_stress_training_gb300 import frames as FR


def test_frame_filename_follows_the_reference():
    name = FR.frame_filename("out/seq", 42)
    stem = "out/seq/h5_f_0000000042"
    assert name == stem + (".h5" if FR.h5py_module() is not None else ".npz")


def test_split_frame_buffer_layout():
    n = 5
    buf = np.arange(34 * n, dtype=np.float32)
    a = FR.split_frame_buffer(buf, n)
    shapes = {"x": (3, n), "q": (3, n), "masses": (1, n), "f_tensor": (9, n), "stress": (6, n), "v": (3, n),
              "C": (9, n)}
    assert {k: v.shape for k, v in a.items()} == shapes
    assert a["x"][0, 0] == 0 and a["q"][0, 0] == 3 * n and a["masses"][0, 0] == 6 * n
    assert a["f_tensor"][0, 0] == 7 * n and a["stress"][0, 0] == 16 * n and a["v"][0, 0] == 22 * n
    assert a["C"][8, n - 1] == 34 * n - 1


def test_stress_components_round_trip():
    rng = np.random.default_rng(0)
    S = rng.normal(size=(7, 3, 3)).astype(np.float32)
    S = S + np.swapaxes(S, 1, 2)
    comps = S.reshape(7, 9)[:, list(FR.STRESS_COMPONENTS)]      # the writer's selection (:383)
    assert np.array_equal(FR.stress_from_components(comps), S)  # the reader's expansion (:283-292)


def test_stress_component_order_is_the_references():
    """Stated independently of the library's own index table: the six stored
    components are [xx, xy, xz, yy, yz, zz] (mpm_solver_warp.py:383 keeps
    flattened indices 0, 1, 2, 4, 5, 8), one row per component, (6, n)."""
    T = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 5.0], [3.0, 5.0, 6.0]], np.float32)
    comps = T.reshape(1, 9)[:, list(FR.STRESS_COMPONENTS)]
    assert comps.tolist() == [[1.0, 2.0, 3.0, 4.0, 5.0, 6.0]]
    n = 3
    buf = np.zeros(34 * n, np.float32)
    buf[16 * n:22 * n] = np.repeat(np.arange(1.0, 7.0, dtype=np.float32), n)  # as the export kernel lays it out
    assert FR.split_frame_buffer(buf, n)["stress"][:, 0].tolist() == [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]
    assert np.array_equal(FR.stress_from_components(comps)[0], T)


def test_store_round_trip_and_resolve(tmp_path, monkeypatch):
    rng = np.random.default_rng(1)
    data = {"x": rng.random((3, 4)).astype(np.float32), "time": np.array([[0.25]]),
            "mu": np.ones((1, 4)) * 30.0}
    path = str(tmp_path / "h5_f_0000000001.npz")
    FR.write_frame(path, data)
    back = FR.read_frame(path)
    assert list(back) == list(data)
    for k in data:
        assert back[k].dtype == data[k].dtype and np.array_equal(back[k], data[k])
    monkeypatch.chdir(tmp_path)
    assert FR.resolve("/h5_f_0000000001.npz") == os.getcwd() + "/h5_f_0000000001.npz"  # cwd + name, as there
    assert FR.resolve(path) == path
    with pytest.raises(FileNotFoundError):
        FR.resolve("/missing.h5")


def test_obj_lines_match_the_reference_format():
    pts = np.array([[0.5, 0.25, 0.125], [1.0 / 3.0, 0.1, 2.0]], np.float32)
    text = FR.obj_lines(pts, [(0.0, 0.0, 0.0), (np.float32(0.5), 0, 0)])
    assert text == "v 0.5 0.25 0.125 0.0 0.0 0.0\nv 0.33333334 0.1 2.0 0.5 0 0\n"


def test_scene_json_round_trip(tmp_path):
    from reduced_mpm_stress_training_gb300 import scenarios as S

    scenes = S.batch_64(n_scenes=5) + [S.sand_column_1m(), S.metal_block_1m()]
    path = str(tmp_path / "scenes.json")
    S.save_scenes(path, scenes)
    back = S.load_scenes(path)
    assert back == scenes
    x_back, x_orig = back[0].particles()[0], scenes[0].particles()[0]   # same seeded particles
    assert np.array_equal(x_back, x_orig)
    S.save_scenes(path, scenes[0])
    assert S.load_scenes(path) == scenes[0]
    with pytest.raises(TypeError):
        S.scene_from_dict(dict(S.scene_to_dict(scenes[0]), unknown=1))
