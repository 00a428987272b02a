"""The C-ABI library loads, exports every entry point include/proland_gb300.h
declares, and its host-side helpers agree with the oracle (no GPU needed)."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(tp_\w+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol(product):
    lib = product.lib()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_no_device_is_reported_not_faked(product):
    # on a machine without a GPU the storage refuses to be created (no CPU fallback)
    if product.device_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(product.TPError) as e:
        product.TileStorage(101, 3, 4)
    assert e.value.code == product.TP_E_NO_DEVICE


@pytest.mark.parametrize("W", [101, 197, 37])
def test_dem_noise_table_matches_oracle(product, oracle_lib, W):
    a = product.dem_noise(W)
    b = oracle_lib.dem_noise(W)
    assert a.shape == (6, W, W)
    assert np.array_equal(a, b)


def test_noise_table_edges_mirror(product):
    """Border bands are written twice, mirrored, so neighbouring tiles match."""
    W = 101
    t = product.dem_noise(W)
    for layer in range(6):
        n = t[layer]
        for h in range(5, W // 2 + 1):
            assert n[2, h] == n[2, W - 1 - h]


def test_cnoise_matches_oracle(product, oracle_lib):
    rng = np.random.default_rng(0)
    pts = rng.uniform(-300, 3000, (500, 2)).astype(np.float32)
    for x, y in pts:
        assert product.cnoise(x, y) == oracle_lib.cnoise(x, y)


def test_noise_select_matches_oracle(product, oracle_lib):
    rng = np.random.default_rng(1)
    for face in range(0, 7):
        for _ in range(60):
            level = int(rng.integers(0, 14))
            tx, ty = (int(v) for v in rng.integers(0, 1 << level, 2))
            assert product.noise_select(face, level, tx, ty) == oracle_lib.noise_select(face, level, tx, ty)
        # the edge cases of the face-continuous parameterisation
        for level in (0, 1, 5):
            o = 1 << level
            for tx, ty in [(0, 0), (o - 1, 0), (0, o - 1), (o - 1, o - 1)]:
                assert product.noise_select(face, level, tx, ty) == oracle_lib.noise_select(face, level, tx, ty)


def test_bad_arguments_return_codes(product):
    lib = product.lib()
    assert lib.tp_storage_create(3, 1, 1, 1, None) == product.TP_E_BAD_ARG
    assert lib.tp_dem_noise(5, None) == product.TP_E_BAD_ARG
    assert lib.tp_last_error()


@pytest.mark.parametrize("D,level,tx,ty", [(12.72e6, 0, 0, 0), (12.72e6, 3, 5, 2), (12.72e6, 12, 1000, 3000), (100000.0, 2, 1, 3)])
def test_sphere_frame_matches_oracle(product, oracle_lib, D, level, tx, ty):
    a = product.sphere_frame(D, level, tx, ty)
    f = oracle_lib.sphere_frame(D, level, tx, ty)
    b = np.concatenate([np.array(f.C), np.array(f.N), np.array(f.L), np.array(f.W2T), [f.R, f.size]]).astype(np.float32)
    assert np.array_equal(a, b)
