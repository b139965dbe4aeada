"""Seeded workloads for the learned layout selector (config 5).

Each workload: dim in {1, 2, 3}; modes 2^6..2^12 per axis, capped so the fine
grid holds at most 2^25 cells; M log-uniform in 1e4..1e8; FP32 or FP64; tol
in {1e-3, 1e-6, 1e-9}; type 1 or 2; point distribution uniform, Gaussian
clusters (1-8 centres, sigma log-uniform in 0.005..1), half uniform and half
clustered, radial (spokes through the centre; 1D: uniform), or a worst case
with every point inside one 8-cell box.  FP32 workloads draw tol = 1e-9 as
1e-6, and M is capped so that M * ns^dim <= 1.2e10 kernel taps (the sweep times
twelve layouts per workload).  Points are generated on the device
from a seeded generator.
"""
from __future__ import annotations

import math

import numpy as np

KINDS = ("uniform", "clusters", "radial", "onebin", "mixed")
MAX_CELLS = 1 << 25
MAX_TAPS = 1.2e10     # M * ns^dim cap: the 3D 3.2e7-point workloads fit, the worst case stays ~0.1 s


def spec(i: int, seed: int = 20261203) -> dict:
    rng = np.random.default_rng(seed + 7919 * i)
    dim = int(rng.integers(1, 4))
    single = bool(rng.integers(0, 2))
    tol = float(rng.choice([1e-3, 1e-6, 1e-9]))
    if single and tol < 1e-6:
        tol = 1e-6        # below FP32's reach; the library would clamp it
    ntype = int(rng.integers(1, 3))
    kind = KINDS[int(rng.integers(0, len(KINDS)))]
    while True:
        modes = [int(2 ** rng.uniform(6, 12)) for _ in range(dim)]
        if np.prod([2 * m + 32 for m in modes]) <= MAX_CELLS:
            break
    M = int(round(10 ** rng.uniform(4, 8)))
    ns = max(2, math.ceil(-math.log10(tol / 10)))
    M = min(M, int(MAX_TAPS // ns ** dim))
    return {"i": i, "dim": dim, "single": single, "tol": tol, "type": ntype, "kind": kind,
            "modes": modes, "M": M, "sigma": float(10 ** rng.uniform(math.log10(0.005), 0)),
            "nclusters": int(rng.integers(1, 9)), "pseed": int(rng.integers(0, 2 ** 31 - 1))}


def points(s: dict, device):
    """Device coordinates (library axis order) for workload s."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(s["pseed"])
    dt = torch.float32 if s["single"] else torch.float64
    M, dim = s["M"], s["dim"]
    two_pi = 2 * math.pi

    def unif(n):
        return (torch.rand(n, generator=g, device=device, dtype=torch.float64) * two_pi - math.pi)

    if s["kind"] == "uniform" or (s["kind"] == "radial" and dim == 1):
        pts = [unif(M) for _ in range(dim)]
    elif s["kind"] == "mixed":  # half uniform, half in Gaussian clusters
        k = s["nclusters"]
        h = M // 2
        centres = torch.rand(k, dim, generator=g, device=device, dtype=torch.float64) * two_pi - math.pi
        which = torch.randint(0, k, (M - h,), generator=g, device=device)
        pts = []
        for d in range(dim):
            x = centres[which, d] + s["sigma"] * torch.randn(M - h, generator=g, device=device,
                                                              dtype=torch.float64)
            pts.append(torch.cat([unif(h), torch.remainder(x + math.pi, two_pi) - math.pi]))
    elif s["kind"] == "clusters":
        k = s["nclusters"]
        centres = torch.rand(k, dim, generator=g, device=device, dtype=torch.float64) * two_pi - math.pi
        which = torch.randint(0, k, (M,), generator=g, device=device)
        pts = []
        for d in range(dim):
            x = centres[which, d] + s["sigma"] * torch.randn(M, generator=g, device=device,
                                                              dtype=torch.float64)
            pts.append(torch.remainder(x + math.pi, two_pi) - math.pi)
    elif s["kind"] == "radial":
        spokes = max(1, int(round(math.sqrt(M / 4))))
        samples = max(1, M // spokes)
        r = torch.linspace(-math.pi, math.pi, samples + 1, device=device, dtype=torch.float64)[:-1]
        if dim == 2:
            th = torch.arange(spokes, device=device, dtype=torch.float64) * math.pi * (3 - math.sqrt(5))
            dirs = [torch.cos(th), torch.sin(th)]
        else:
            v = torch.randn(spokes, 3, generator=g, device=device, dtype=torch.float64)
            v = v / v.norm(dim=1, keepdim=True)
            dirs = [v[:, 0], v[:, 1], v[:, 2]]
        pts = [(dd[:, None] * r[None, :]).reshape(-1) for dd in dirs]
        M = pts[0].numel()
        s["M"] = M
    else:  # every point inside one 8-cell box
        pts = []
        for d in range(dim):
            nf = 2 * s["modes"][d]
            a = float(torch.rand(1, generator=g, device=device).item()) * two_pi - math.pi
            w = two_pi * 8 / nf
            pts.append(torch.remainder(a + w * torch.rand(M, generator=g, device=device,
                                                          dtype=torch.float64) + math.pi, two_pi)
                       - math.pi)
    return [p.to(dt).contiguous() for p in pts]


def heuristic_class(s: dict) -> int:
    """Layout class of the reference's default options: type 1 runs method 2,
    type 2 method 1, both with the medium (default) bins and cap 1024."""
    return 6 if s["type"] == 1 else 1
