"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations (the reference ships no dataset; its own generators,
host/host/generator.cpp, draw uniform keys with glibc rand()).

All generators use torch so that the large configurations can be generated on
the GPU; a given (seed, device) pair always yields the same data.

  config 0  filter        : key uniform [0, 2^31), payload uniform [0, 1000)
  config 1  group-by      : key Zipf(s) over G groups, rank -> key through a
                            seeded permutation of 0..G-1; value, value2
                            uniform [0, 1000)
  config 2  join          : R keys = seeded permutation of 0..nR-1, payload
                            uniform [0, 1000); S keys 80 % uniform over R's
                            keys, 20 % uniform over [2^24, 2^31); S payload
                            uniform [0, 1000)
  config 4  skewed join   : keys from 8 Gaussians (sigma 2^20) plus a 5 %
                            Zipf(1.2) heavy-hitter component
"""
from __future__ import annotations

import torch


def _gen(seed: int, device) -> torch.Generator:
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    return g


def uniform_i32(n: int, lo: int, hi: int, seed: int, device="cpu") -> torch.Tensor:
    """int32 uniform in [lo, hi)."""
    return torch.randint(lo, hi, (n,), generator=_gen(seed, device), dtype=torch.int64,
                         device=device).to(torch.int32)


def config0_filter(n: int = 1 << 24, seed: int = 0, device="cpu"):
    key = uniform_i32(n, 0, 2 ** 31, seed, device)
    pay = uniform_i32(n, 0, 1000, seed + 1, device)
    # predicate key < 2^31 / 10  ->  inclusive range [INT32_MIN, 214748363]
    return {"key": key, "payload": pay, "lo": -(2 ** 31), "hi": 214748363}


def zipf_ranks(n: int, groups: int, s: float, seed: int, device="cpu") -> torch.Tensor:
    """Ranks in [0, groups) with P(rank=k) proportional to 1/(k+1)^s (inverse CDF)."""
    k = torch.arange(1, groups + 1, dtype=torch.float64, device=device)
    w = k.pow(-s)
    cdf = torch.cumsum(w, 0)
    cdf = cdf / cdf[-1]
    u = torch.rand(n, generator=_gen(seed, device), dtype=torch.float64, device=device)
    r = torch.searchsorted(cdf, u)
    return r.clamp_(max=groups - 1)


def config1_groupby(n: int = 1 << 26, groups: int = 1 << 20, s: float = 1.0, seed: int = 0,
                    device="cpu"):
    ranks = zipf_ranks(n, groups, s, seed, device)
    perm = torch.randperm(groups, generator=_gen(seed + 7, device), device=device)
    key = perm[ranks].to(torch.int32)
    val = uniform_i32(n, 0, 1000, seed + 1, device)
    val2 = uniform_i32(n, 0, 1000, seed + 2, device)
    # fused predicate value2 < 500 -> [INT32_MIN, 499]
    return {"key": key, "val": val, "val2": val2, "lo2": -(2 ** 31), "hi2": 499, "groups": groups}


def config2_join(nR: int = 1 << 24, nS: int = 1 << 28, seed: int = 0, device="cpu",
                 hit_rate: float = 0.8):
    rkey = torch.randperm(nR, generator=_gen(seed, device), device=device).to(torch.int32)
    rpay = uniform_i32(nR, 0, 1000, seed + 1, device)
    g = _gen(seed + 2, device)
    inside = torch.rand(nS, generator=g, device=device) < hit_rate
    k_in = torch.randint(0, nR, (nS,), generator=g, device=device, dtype=torch.int64)
    k_out = torch.randint(max(nR, 1 << 24), 2 ** 31, (nS,), generator=g, device=device,
                          dtype=torch.int64)
    skey = torch.where(inside, k_in, k_out).to(torch.int32)
    del k_in, k_out, inside
    spay = uniform_i32(nS, 0, 1000, seed + 3, device)
    # filter S.payload < 300 -> [INT32_MIN, 299]
    return {"rkey": rkey, "rpay": rpay, "skey": skey, "spay": spay, "slo": -(2 ** 31), "shi": 299}


def skewed_keys(n: int, seed: int, device="cpu", heavy_frac: float = 0.05,
                sample_seed: int | None = None) -> torch.Tensor:
    """8 Gaussians (means uniform over int32, sigma 2^20) + Zipf(1.2) heavy hitters.

    `seed` fixes the mixture (means, heavy keys); `sample_seed` (default
    `seed`) the draws, so that two sides can share one mixture."""
    g = _gen(seed, device)
    means = torch.randint(-(2 ** 31) + (1 << 24), 2 ** 31 - (1 << 24), (8,), generator=g,
                          device=device, dtype=torch.int64).to(torch.float64)
    hkeys = torch.randint(-(2 ** 31), 2 ** 31 - 1, (1 << 16,), generator=g, device=device,
                          dtype=torch.int64)
    gs = _gen(seed if sample_seed is None else sample_seed + 1_000_003, device)
    comp = torch.randint(0, 8, (n,), generator=gs, device=device)
    x = means[comp] + torch.randn(n, generator=gs, device=device, dtype=torch.float64) * float(1 << 20)
    x = x.round().clamp(-(2 ** 31), 2 ** 31 - 1).to(torch.int64)
    heavy = torch.rand(n, generator=gs, device=device) < heavy_frac
    hk = zipf_ranks(n, 1 << 16, 1.2, (seed if sample_seed is None else sample_seed) + 11, device)
    x = torch.where(heavy, hkeys[hk], x)
    return x.to(torch.int32)


def config4_skewed(nR: int = 1 << 25, nS: int = 1 << 28, seed: int = 0, device="cpu"):
    """Skewed join: R = nR distinct keys drawn from the mixture (a unique
    build side, as in config 2), S = nS keys drawn from the same mixture
    (heavy hitters included), payloads uniform [0, 1000), filter S.payload < 300."""
    want = nR
    draw = int(nR * 1.6) + 1024
    while True:
        cand = torch.unique(skewed_keys(draw, seed, device, sample_seed=seed + 1))
        if cand.numel() >= want:
            break
        draw *= 2
    perm = torch.randperm(cand.numel(), generator=_gen(seed + 2, device), device=device)[:want]
    rkey = cand[perm].to(torch.int32)
    del cand, perm
    rpay = uniform_i32(nR, 0, 1000, seed + 3, device)
    skey = skewed_keys(nS, seed, device, sample_seed=seed + 4)
    spay = uniform_i32(nS, 0, 1000, seed + 5, device)
    return {"rkey": rkey, "rpay": rpay, "skey": skey, "spay": spay, "slo": -(2 ** 31), "shi": 299}


def records(key: torch.Tensor, payload: torch.Tensor | None = None) -> torch.Tensor:
    """Reference Records (n, 2) int32 {x = payload or row id, y = key}."""
    n = key.numel()
    x = torch.arange(n, dtype=torch.int32, device=key.device) if payload is None else payload
    return torch.stack([x.to(torch.int32), key.to(torch.int32)], dim=1).contiguous()
