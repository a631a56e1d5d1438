"""Seeded synthetic point clouds with the shapes of the five benchmark workloads.

No public dataset is involved; every generator draws from
``np.random.default_rng(seed)`` and returns float32.

  single-4k       4,096 x 3 uniform [0,1)^3, K=1,024, start 0 (vanilla FPS)
  gmm-1m          1,048,576 x 3, mixture of 64 isotropic Gaussians (means
                  U[0,100)^3, sigma U[0.5,5]), K=16,384, start 0, kd-line h=7
  batched-256     256 clouds, N log-uniform in [1,024, 131,072], U[0,1)^3 with a
                  per-cloud per-axis scale U[0.1,10], K=N//4, start 0
  served          Poisson arrivals at 2,000 req/s for 10 s; N log-uniform in
                  [4,096, 2,097,152]; points on 16 random spheres (centres
                  U[0,100)^3, radius U[1,10]) plus 1% uniform outliers in their
                  bounding box; K uniform in [N/16, N/4]; start uniform in [0,N)
  large-16m       16,777,216 x 6: xyz U[0,1000)^3 + 3 channels U[0,1),
                  K=65,536, start 0 (vanilla and kd-line h=9)
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEEDS = {"single-4k": 0, "gmm-1m": 1, "batched-256": 2, "served": 3, "large-16m": 4}


def uniform_cloud(n: int, d: int = 3, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.random((n, d), dtype=np.float64).astype(np.float32)


def gmm_cloud(n: int, n_comp: int = 64, seed: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    means = rng.random((n_comp, 3)) * 100.0
    sigma = rng.uniform(0.5, 5.0, n_comp)
    lab = rng.integers(0, n_comp, n)
    pts = means[lab] + rng.standard_normal((n, 3)) * sigma[lab, None]
    return pts.astype(np.float32)


def scaled_box_cloud(rng: np.random.Generator, n: int) -> np.ndarray:
    scale = rng.uniform(0.1, 10.0, 3)
    return (rng.random((n, 3)) * scale).astype(np.float32)


def batched_clouds(n_clouds: int = 256, lo: int = 1024, hi: int = 131072, seed: int = 2):
    """[(points, K)] for the batched workload (K = N // 4, start 0)."""
    rng = np.random.default_rng(seed)
    sizes = np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), n_clouds))).astype(np.int64)
    out = []
    for n in sizes:
        pts = scaled_box_cloud(rng, int(n))
        out.append((pts, int(n) // 4))
    return out


def sphere_cloud(rng: np.random.Generator, n: int, n_spheres: int = 16, outlier_frac: float = 0.01):
    centres = rng.random((n_spheres, 3)) * 100.0
    radius = rng.uniform(1.0, 10.0, n_spheres)
    n_out = int(round(n * outlier_frac))
    n_surf = n - n_out
    lab = rng.integers(0, n_spheres, n_surf)
    v = rng.standard_normal((n_surf, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    surf = centres[lab] + v * radius[lab, None]
    lo = (centres - radius[:, None]).min(axis=0)
    hi = (centres + radius[:, None]).max(axis=0)
    outl = lo + rng.random((n_out, 3)) * (hi - lo)
    pts = np.concatenate([surf, outl]).astype(np.float32)
    return pts[rng.permutation(n)]


@dataclass
class Request:
    """One served request; its points come from its own seed, so a request
    stream can be drawn without holding every cloud in memory."""
    arrival_s: float
    n: int
    k: int
    start: int
    seed: int

    def points(self) -> np.ndarray:
        return sphere_cloud(np.random.default_rng(self.seed), self.n)


def request_stream(rate: float = 2000.0, duration_s: float = 10.0, lo: int = 4096,
                   hi: int = 2097152, seed: int = 3, max_requests: int | None = None):
    """Yield the served workload's requests in arrival order (points are
    generated by Request.points)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    i = 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration_s or (max_requests is not None and i >= max_requests):
            return
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        k = int(rng.integers(n // 16, n // 4 + 1))
        start = int(rng.integers(0, n))
        yield Request(t, n, k, start, int(rng.integers(0, 2**63)))
        i += 1


def large_cloud(n: int = 16_777_216, seed: int = 4) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = np.empty((n, 6), np.float32)
    out[:, :3] = rng.random((n, 3), dtype=np.float32) * 1000.0
    out[:, 3:] = rng.random((n, 3), dtype=np.float32)
    return out
