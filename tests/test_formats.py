"""seed/{name}.json and kernels/{name}_{n}.bin through the C ABI (CPU only).

The C++ loaders (config_io.cpp) must agree with the oracle's restatement of
ml-rs/config.rs:32-125, including the c0/c1 swap (config.rs:40) and the
spectral zero-padding resample (config.rs:81-116), and must return error
codes where the reference panics.
"""
import json
import os

import numpy as np
import pytest

from cella_nova_gb300 import CellaError, load_config, load_kernels
from cella_nova_gb300.creature import make_creature, write_creature, write_kernels_bin
from oracle import oracle as O


@pytest.fixture
def creature_files(tmp_path):
    cr = make_creature(32, 3, seed=9, radius=(3, 7), seed_box=16, temp=1.25)
    js, kb = write_creature(str(tmp_path), "crit", cr)
    return cr, js, kb


def test_config_matches_oracle_loader(creature_files):
    cr, js, _ = creature_files
    got = load_config(js)
    ref = O.load_config_np(js)
    assert got["seed_size"] == 32 and got["num_channels"] == 3 and got["num_kernels"] == 9
    np.testing.assert_array_equal(got["c0"], ref["c0"])
    np.testing.assert_array_equal(got["c1"], ref["c1"])
    np.testing.assert_array_equal(got["c0"], cr.c0)      # orchestrator order after swap
    np.testing.assert_array_equal(got["seed_channels"].reshape(3, 32, 32), ref["seed"])
    np.testing.assert_array_equal(got["growth_mu"], ref["mu"])
    np.testing.assert_array_equal(got["growth_sigma"], ref["sigma"])
    np.testing.assert_array_equal(got["growth_weights"], ref["weights"])
    assert abs(got["temp"] - 1.25) < 1e-7


def test_reference_style_json_without_extras(tmp_path):
    """The reference generator's key set only (generate_kernel_json.py:202-212)."""
    n, C, K = 16, 1, 1
    data = {"seed_size": n, "num_channels": C, "num_kernels": K,
            "seed_channels": [[0.5] * (n * n)], "c0": [0], "c1": [0],
            "growth_mu": [0.15], "growth_sigma": [0.015], "growth_weights": [1.0],
            "global_r": 10.0, "radii": [0.25], "widths": [0.03]}
    p = tmp_path / "ref.json"
    p.write_text(json.dumps(data, indent=2))
    got = load_config(str(p))
    assert got["temp"] == 1.0
    assert got["seed_channels"].shape == (1, n * n)


def test_kernels_same_size_and_resampled(creature_files):
    cr, _, kb = creature_files
    same = load_kernels(kb, cr.K, 32)
    np.testing.assert_array_equal(same, cr.kspec)
    for target in (64, 128):
        got = load_kernels(kb, cr.K, target)
        ref = O.load_kernels_np(kb, cr.K, target)
        np.testing.assert_array_equal(got, ref)


def test_kernels_larger_than_target_rejected(creature_files):
    cr, _, kb = creature_files
    with pytest.raises(CellaError, match="UNSUPPORTED"):
        load_kernels(kb, cr.K, 16)


def test_truncated_kernel_file(tmp_path):
    p = tmp_path / "bad.bin"
    write_kernels_bin(str(p), np.ones((2, 16, 16), np.complex64))
    raw = p.read_bytes()
    p.write_bytes(raw[:-8])
    with pytest.raises(CellaError, match="FORMAT"):
        load_kernels(str(p), 2, 16)


def test_missing_files_and_fields(tmp_path):
    with pytest.raises(CellaError, match="IO"):
        load_config(str(tmp_path / "nope.json"))
    with pytest.raises(CellaError, match="IO"):
        load_kernels(str(tmp_path / "nope.bin"), 1, 16)
    p = tmp_path / "partial.json"
    p.write_text(json.dumps({"seed_size": 4, "num_channels": 1, "num_kernels": 1}))
    with pytest.raises(CellaError, match="FORMAT"):
        load_config(str(p))


@pytest.mark.parametrize("mutate,msg", [
    (lambda d: d.update(c0=[5]), "channel index"),
    (lambda d: d.update(growth_mu=[0.1, 0.2]), "num_kernels"),
    (lambda d: d["seed_channels"][0].pop(), "seed channel"),
    (lambda d: d.update(num_channels=2), "seed channels"),
])
def test_inconsistent_config_rejected(tmp_path, mutate, msg):
    n = 4
    d = {"seed_size": n, "num_channels": 1, "num_kernels": 1,
         "seed_channels": [[0.0] * (n * n)], "c0": [0], "c1": [0],
         "growth_mu": [0.1], "growth_sigma": [0.01], "growth_weights": [1.0]}
    mutate(d)
    p = tmp_path / "bad.json"
    p.write_text(json.dumps(d))
    with pytest.raises(CellaError, match=msg):
        load_config(str(p))


def test_malformed_json(tmp_path):
    p = tmp_path / "broken.json"
    p.write_text('{"seed_size": 4, "num_channels": ')
    with pytest.raises(CellaError, match="FORMAT"):
        load_config(str(p))
    assert os.path.exists(p)


# -- binary twin of the seed JSON ---------------------------------------------

def _same_config(a, b):
    for key in ("seed_size", "num_channels", "num_kernels"):
        assert a[key] == b[key], key
    for key in ("seed_channels", "c0", "c1", "growth_mu", "growth_sigma", "growth_weights"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)
    assert a["temp"] == b["temp"]


def test_seed_bin_round_trip_equals_json(creature_files, tmp_path):
    from cella_nova_gb300.orchestrator import save_config_bin
    cr, js, _ = creature_files
    from_json = load_config(js)
    path = tmp_path / "crit.seedbin"
    save_config_bin(path, from_json)
    _same_config(load_config(path), from_json)
    # bit-exact f64 seeds, JSON-order channel fields
    raw = path.read_bytes()
    assert raw[:8] == b"CNSEED01"
    assert len(raw) == 24 + 5 * 4 * cr.K + 4 + 8 * cr.C * cr.n * cr.n   # 9 kernels: 4 pad bytes


def test_seed_bin_python_writer_matches_c_writer(creature_files, tmp_path):
    from cella_nova_gb300.creature import write_seed_bin
    from cella_nova_gb300.orchestrator import save_config_bin
    cr, js, _ = creature_files
    a, b = tmp_path / "py.seedbin", tmp_path / "c.seedbin"
    write_seed_bin(str(a), cr)
    save_config_bin(b, load_config(js))
    assert a.read_bytes() == b.read_bytes()


def test_seed_bin_rejects_bad_files(creature_files, tmp_path):
    from cella_nova_gb300.creature import write_seed_bin
    cr, _, _ = creature_files
    good = tmp_path / "g.seedbin"
    write_seed_bin(str(good), cr)
    raw = good.read_bytes()
    cases = {
        "truncated": raw[:-8],
        "index": raw[:24] + (7).to_bytes(4, "little") + raw[28:],   # channel 7 of 3
    }
    for name, data in cases.items():
        p = tmp_path / f"{name}.seedbin"
        p.write_bytes(data)
        with pytest.raises(CellaError) as e:
            load_config(p)
        assert e.value.code == -6, name     # CG_ERR_FORMAT


def test_setup_simulation_accepts_seed_bin(creature_files, tmp_path):
    from cella_nova_gb300.creature import write_seed_bin
    cr, js, _ = creature_files
    p = tmp_path / "s.seedbin"
    write_seed_bin(str(p), cr)
    _same_config(load_config(p), load_config(js))
