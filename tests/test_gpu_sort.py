"""GPU parity: sort_indices gives the reference runtime's exact permutation
(stable LSD radix on signed 8-bit digits), and gather."""
import glob
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _sort(hc, keys_np, dev, key_bits=None):
    keys = torch.from_numpy(np.ascontiguousarray(keys_np, dtype=np.int64)).to(dev)
    perm = torch.full_like(keys, -1)
    hc.sort_indices(keys, perm, key_bits=key_bits)
    hc.check(hc.device_check())
    return perm.cpu().numpy()


def test_known_answer(hc, dev):
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        c = json.load(f)["sort_indices_gather_test"]
    assert _sort(hc, c["keys"], dev).tolist() == c["perm"]


def test_reference_runtime_vectors(hc, dev):
    for f in sorted(glob.glob(os.path.join(GOLDEN, "witness_sort_*.npz"))):
        z = np.load(f)
        assert np.array_equal(_sort(hc, z["keys"], dev), z["perm"]), f


@pytest.mark.parametrize("n", [1, 2, 33, 4095, 4096, 4097, 100_003, 1 << 20])
@pytest.mark.parametrize("hi", [1, 3, 256, 1 << 20, 1 << 36, 1 << 62])
def test_random_keys_match_oracle(hc, orc, dev, n, hi):
    rng = np.random.default_rng(n * 7 + hi % 1000)
    keys = rng.integers(0, hi, size=n, dtype=np.int64) if hi > 1 else np.zeros(n, dtype=np.int64)
    assert np.array_equal(_sort(hc, keys, dev), orc.sort_indices(keys))


def test_negative_keys_follow_runtime_digits(hc, orc, dev):
    # the runtime derives the pass count from the largest key and takes digits
    # of the signed key; negative keys sort by those low digits only
    rng = np.random.default_rng(11)
    keys = rng.integers(-(1 << 20), 1 << 12, size=20000, dtype=np.int64)
    assert np.array_equal(_sort(hc, keys, dev), orc.sort_indices(keys))


def test_key_bits_variant(hc, orc, dev):
    rng = np.random.default_rng(12)
    keys = rng.integers(0, 1 << 36, size=300_000, dtype=np.int64)
    assert np.array_equal(_sort(hc, keys, dev, key_bits=36), orc.sort_indices(keys))


def test_packed_coo_keys_full_size(hc, orc, dev):
    """Packed row*ncols+col keys of a 2^18 x 2^18 instance (the batched workload's largest)."""
    rng = np.random.default_rng(13)
    n = 3_200_000
    keys = rng.integers(0, 1 << 18, size=n, dtype=np.int64) * (1 << 18) + rng.integers(0, 1 << 18, size=n)
    assert np.array_equal(_sort(hc, keys, dev), orc.sort_indices(keys))


def test_gather(hc, dev):
    rng = np.random.default_rng(14)
    src = rng.integers(-100, 100, size=1000, dtype=np.int64)
    perm = rng.integers(0, 1000, size=5000, dtype=np.int64)
    d_perm = torch.from_numpy(perm).to(dev)
    for dtype, conv in ((torch.int64, np.int64), (torch.float64, np.float64), (torch.int32, np.int32)):
        s = torch.from_numpy(src.astype(conv)).to(dev)
        out = torch.empty(5000, dtype=dtype, device=dev)
        hc.gather(d_perm, s, out)
        assert np.array_equal(out.cpu().numpy(), src.astype(conv)[perm])
    bad = torch.tensor([0, 1000], dtype=torch.int64, device=dev)
    out = torch.zeros(2, dtype=torch.int64, device=dev)
    hc.gather(bad, torch.from_numpy(src).to(dev), out)
    assert hc.device_check() == hc.ERR_BOUNDS
