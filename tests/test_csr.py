"""Sparse-key CSR rank-LUT (CsrBase of sparse_engine.hpp:70-102, build_csr_base of
sparse_engine.hpp:287-360).

CPU: the oracle reproduces the golden vectors answered by the reference's own
CsrBase::rank / CsrBase::range (tests/golden/make_csr_golden.py).  GPU: the device
build (radix sort + run-length + bucket LUT) and lookups reproduce the golden vectors
at several LUT budgets, match the oracle bit for bit on random 40-bit keys (both the
low-bits probe and the full-key probe), and at the configured size satisfy the
size-independent properties (sorted distinct keys, amount total, present keys rank
to their own index)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "csr_golden.npz")
CASES = sorted({k.rsplit("_", 1)[0] for k in GOLD.files if k.endswith("_C")})


def golden(name):
    g = {k[len(name) + 1:]: GOLD[k] for k in GOLD.files if k.startswith(name + "_")}
    g["C"] = int(g["C"][0])
    return g


def key_bits_for(C: int) -> int:
    return max(1, int(C - 1).bit_length())


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_csrbase(oracle_mod, name):
    g = golden(name)
    uk, pre = oracle_mod.csr_build(g["cls"].astype(np.uint64), g["amt"])
    q = g["q"].astype(np.uint64)
    pt = oracle_mod.csr_point(uk, q[:, 0])
    rank = np.where(pt >= 0, pt, -pt - 1)
    np.testing.assert_array_equal(rank, g["rank_lo"])
    rg = oracle_mod.csr_range(uk, pre, q)
    np.testing.assert_array_equal(rg[:, 0], g["rank_hi"] - g["rank_lo"])
    np.testing.assert_array_equal(rg[:, 1], g["range"])


def test_oracle_properties_random_keys(oracle_mod):
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 1 << 40, 5000, dtype=np.uint64)
    keys = np.concatenate([keys, keys[:1000]])
    amt = rng.integers(-1000, 1000, keys.size, dtype=np.int64)
    uk, pre = oracle_mod.csr_build(keys, amt)
    np.testing.assert_array_equal(uk, np.unique(keys))
    assert pre[-1] == amt.sum()
    pt = oracle_mod.csr_point(uk, uk)
    np.testing.assert_array_equal(pt, np.arange(uk.size))


# ------------------------------------------------------------------------------ GPU
def _index(bw, torch, keys, amounts, key_bits, budget):
    k = torch.from_numpy(np.ascontiguousarray(keys).view(np.int64)).cuda()
    a = torch.from_numpy(np.ascontiguousarray(amounts)).cuda()
    return bw.CsrIndex(k, a, key_bits=key_bits, lut_budget_bytes=budget)


def _u64_cuda(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.uint64).view(np.int64)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("budget", [4, 64, 4096, 1 << 20])
def test_gpu_csr_matches_reference_csrbase(bw, torch_cuda, name, budget):
    torch = torch_cuda
    g = golden(name)
    idx = _index(bw, torch, g["cls"].astype(np.uint64), g["amt"], key_bits_for(g["C"]), budget)
    q = g["q"].astype(np.uint64)
    pt = idx.point(_u64_cuda(torch, q[:, 0].copy())).cpu().numpy()
    rank = np.where(pt >= 0, pt, -pt - 1)
    np.testing.assert_array_equal(rank, g["rank_lo"])
    rg = idx.range(_u64_cuda(torch, q)).cpu().numpy()
    np.testing.assert_array_equal(rg[:, 0], g["rank_hi"] - g["rank_lo"])
    np.testing.assert_array_equal(rg[:, 1], g["range"])


@pytest.mark.gpu
@pytest.mark.parametrize("budget", [1 << 10, 1 << 20, 64 << 20, 256 << 20])
def test_gpu_csr_random_keys_vs_oracle(bw, torch_cuda, oracle_mod, budget):
    # below 64 MiB the 2^40 universe needs buckets wider than 2^16 keys: the full-key
    # probe; from 64 MiB (2^24 buckets) on, the u16 low-bits probe
    torch = torch_cuda
    rng = np.random.default_rng(budget)
    base = rng.integers(0, 1 << 40, 200_000, dtype=np.uint64)
    keys = np.concatenate([base, base[rng.integers(0, base.size, 300_000)]])
    amt = rng.integers(-(1 << 30), 1 << 30, keys.size, dtype=np.int64)
    idx = _index(bw, torch, keys, amt, 40, budget)
    assert (idx.shift <= 16) == (budget >= (64 << 20))
    uk, pre = oracle_mod.csr_build(keys, amt)
    assert idx.count() == uk.size
    dk, dp = idx.arrays()
    np.testing.assert_array_equal(dk.cpu().numpy().view(np.uint64), uk)
    np.testing.assert_array_equal(dp.cpu().numpy(), pre)
    look = np.concatenate([uk[rng.integers(0, uk.size, 50_001)],
                           rng.integers(0, 1 << 40, 50_000, dtype=np.uint64),
                           np.array([0, (1 << 40) - 1, 1 << 40, (1 << 64) - 1], np.uint64)])
    pt = idx.point(_u64_cuda(torch, look)).cpu().numpy()
    np.testing.assert_array_equal(pt, oracle_mod.csr_point(uk, look))
    a, b = rng.permutation(look), rng.permutation(look)
    bounds = np.stack([a, b], axis=1)   # includes hi < lo (negative, as the reference)
    rg = idx.range(_u64_cuda(torch, bounds)).cpu().numpy()
    np.testing.assert_array_equal(rg, oracle_mod.csr_range(uk, pre, bounds))


@pytest.mark.gpu
def test_gpu_csr_empty_and_single(bw, torch_cuda, oracle_mod):
    torch = torch_cuda
    idx = _index(bw, torch, np.zeros(0, np.uint64), np.zeros(0, np.int64), 40, 1 << 16)
    assert idx.count() == 0
    look = np.array([0, 5, 1 << 39], np.uint64)
    np.testing.assert_array_equal(idx.point(_u64_cuda(torch, look)).cpu().numpy(), [-1, -1, -1])
    idx = _index(bw, torch, np.array([7, 7, 7], np.uint64), np.array([1, 2, 3], np.int64), 40, 1 << 16)
    assert idx.count() == 1
    np.testing.assert_array_equal(idx.point(_u64_cuda(torch, np.array([6, 7, 8], np.uint64))).cpu().numpy(),
                                  [-1, 0, -2])
    rg = idx.range(_u64_cuda(torch, np.array([[0, 8], [7, 7], [8, 0]], np.uint64))).cpu().numpy()
    np.testing.assert_array_equal(rg, [[1, 6], [0, 0], [-1, -6]])


@pytest.mark.gpu
def test_gpu_csr_configured_size_properties(bw, torch_cuda, oracle_mod):
    """10M distinct keys, 20M events, lookups sampled: the full-size build and a
    sample of its lookups against the oracle."""
    torch = torch_cuda
    w = bw.workloads.csr_lut(0, 1.0, lookups=2_000_000)
    idx = _index(bw, torch, w.keys, w.amounts, w.key_bits, 256 << 20)
    assert idx.count() == w.n_distinct
    dk, dp = idx.arrays()
    dk = dk.cpu().numpy().view(np.uint64)
    assert np.all(dk[1:] > dk[:-1])
    assert int(dp[-1].item()) == int(w.amounts.sum())
    ok, opre = oracle_mod.csr_build(w.keys, w.amounts)
    np.testing.assert_array_equal(dk, ok)
    np.testing.assert_array_equal(dp.cpu().numpy(), opre)
    rng = np.random.default_rng(5)
    s = rng.integers(0, w.n_distinct, 1_000_000)
    np.testing.assert_array_equal(idx.point(_u64_cuda(torch, dk[s])).cpu().numpy(), s)
    j = rng.integers(0, len(w.point), 200_000)
    uk = dk
    pre = dp.cpu().numpy()
    np.testing.assert_array_equal(idx.point(_u64_cuda(torch, w.point[j])).cpu().numpy(),
                                  oracle_mod.csr_point(uk, w.point[j]))
    np.testing.assert_array_equal(idx.range(_u64_cuda(torch, w.ranges[j])).cpu().numpy(),
                                  oracle_mod.csr_range(uk, pre, w.ranges[j]))


@pytest.mark.gpu
def test_gpu_csr_flags_key_outside_universe(bw, torch_cuda):
    """A build key >= 2^key_bits is reported through the status word; lookups on
    that index stay in bounds (their values are unspecified)."""
    torch = torch_cuda
    keys = np.array([1, (1 << 41) + 3, 5, 9, 1 << 39], np.uint64)
    idx = _index(bw, torch, keys, np.ones(keys.size, np.int64), 40, 1 << 12)
    assert idx.status() == 1
    idx.point(_u64_cuda(torch, np.array([0, 1, 5, 9, 1 << 39, 1 << 41], np.uint64)))
    idx.range(_u64_cuda(torch, np.array([[0, 1 << 40], [5, 3]], np.uint64)))
    torch.cuda.synchronize()
    ok = _index(bw, torch, keys[[0, 2, 3, 4]], np.ones(4, np.int64), 40, 1 << 12)
    assert ok.status() == 0
