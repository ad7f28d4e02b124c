"""Seeded synthetic point sets with the shapes of the benchmark workloads.

No public dataset is involved: each generator restates a workload description (sizes,
mixture structure, value distributions) with numpy's PCG64 generator, so a seed fixes the
data bit for bit on any machine.
"""
from __future__ import annotations

import numpy as np


def blobs_with_noise(n: int = 2000, d: int = 10, centers: int = 8, std: float = 1.0,
                     noise_fraction: float = 0.05, seed: int = 42) -> np.ndarray:
    """Isotropic Gaussian blobs (centres uniform in [-10, 10]^d, equal weights) plus uniform
    noise over the bounding box of the blob points; float32 rows in shuffled order."""
    rng = np.random.default_rng(seed)
    n_noise = int(round(n * noise_fraction))
    n_blob = n - n_noise
    c = rng.uniform(-10.0, 10.0, size=(centers, d))
    assign = rng.integers(0, centers, size=n_blob)
    pts = c[assign] + rng.normal(0.0, std, size=(n_blob, d))
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    noise = rng.uniform(lo, hi, size=(n_noise, d))
    x = np.concatenate([pts, noise]).astype(np.float32)
    return x[rng.permutation(n)]


def anisotropic_mixture(n: int = 100_000, d: int = 64, components: int = 50,
                        noise_fraction: float = 0.02, seed: int = 43) -> np.ndarray:
    """Gaussian mixture with random anisotropic covariances Q diag(l) Q^T (l log-uniform in
    [0.1, 2], Q a random rotation), Dirichlet(1) weights, centres uniform in [-10, 10]^d, plus
    uniform noise over the bounding box."""
    rng = np.random.default_rng(seed)
    n_noise = int(round(n * noise_fraction))
    n_mix = n - n_noise
    weights = rng.dirichlet(np.ones(components))
    counts = rng.multinomial(n_mix, weights)
    centres = rng.uniform(-10.0, 10.0, size=(components, d))
    parts = []
    for c in range(components):
        if counts[c] == 0:
            continue
        q, r = np.linalg.qr(rng.normal(size=(d, d)))
        q = q * np.sign(np.diag(r))
        lam = np.exp(rng.uniform(np.log(0.1), np.log(2.0), size=d))
        z = rng.normal(size=(counts[c], d)) * np.sqrt(lam)
        parts.append(centres[c] + z @ q.T)
    pts = np.concatenate(parts)
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    noise = rng.uniform(lo, hi, size=(n_noise, d))
    x = np.concatenate([pts, noise]).astype(np.float32)
    return x[rng.permutation(n)]


def vmf_like(n: int = 500_000, d: int = 128, clusters: int = 100, noise_fraction: float = 0.01,
             kappa_range=(20.0, 200.0), seed: int = 44, chunk: int = 65536) -> np.ndarray:
    """Unit vectors from clusters approximating von Mises-Fisher: sample = normalise(mu + g/sqrt(k))
    with g standard normal, unit mean directions mu and concentration k uniform in kappa_range;
    plus uniformly random unit vectors. (The normalised Gaussian perturbation approximates a vMF
    draw; it is not an exact vMF sampler.)"""
    rng = np.random.default_rng(seed)
    n_noise = int(round(n * noise_fraction))
    n_cl = n - n_noise
    mu = rng.normal(size=(clusters, d))
    mu /= np.linalg.norm(mu, axis=1, keepdims=True)
    kappa = rng.uniform(kappa_range[0], kappa_range[1], size=clusters)
    assign = rng.integers(0, clusters, size=n_cl)
    out = np.empty((n, d), np.float32)
    for a in range(0, n_cl, chunk):
        b = min(n_cl, a + chunk)
        idx = assign[a:b]
        v = mu[idx] + rng.normal(size=(b - a, d)) / np.sqrt(kappa[idx])[:, None]
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        out[a:b] = v
    g = rng.normal(size=(n_noise, d))
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    out[n_cl:] = g
    return out[rng.permutation(n)]


def gaussian_mixture(n: int, d: int, blobs: int, std_range=(0.5, 2.0), seed: int = 0) -> np.ndarray:
    """Isotropic Gaussian blobs with centres uniform in [-10, 10]^d, equal weights and a
    standard deviation per blob uniform in std_range; float32 rows in shuffled order."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-10.0, 10.0, size=(blobs, d))
    std = rng.uniform(std_range[0], std_range[1], size=blobs)
    assign = rng.integers(0, blobs, size=n)
    x = (c[assign] + rng.normal(size=(n, d)) * std[assign, None]).astype(np.float32)
    return x


def fit_request_stream(count: int, seed: int = 46) -> list[dict]:
    """Specifications of a stream of fit requests: n log-uniform in [500, 50000], d drawn from
    {16, 32, 64, 128}, a Gaussian mixture of blobs ~ U{2..30} (std U[0.5, 2], centres
    U[-10, 10]^d); min_samples = 5, min_cluster_size = max(5, n / 200)."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(500), np.log(50000), size=count)).astype(np.int64)
    d = rng.choice([16, 32, 64, 128], size=count)
    blobs = rng.integers(2, 31, size=count)
    return [{"n": int(n[i]), "d": int(d[i]), "blobs": int(blobs[i]), "min_samples": 5,
             "min_cluster_size": max(5, int(n[i]) // 200), "seed": seed * 1_000_003 + i}
            for i in range(count)]


def request_points(spec: dict) -> np.ndarray:
    """The point set of one request specification."""
    return gaussian_mixture(spec["n"], spec["d"], spec["blobs"], seed=spec["seed"])


def repeated_points(n: int = 150_000, d: int = 8, copies: int = 3, seed: int = 3) -> np.ndarray:
    """n // copies uniform points in [0, 1)^d, each repeated `copies` times in a row: every
    kNN row holds exact duplicates and points of other groups, the case where a Borůvka round
    screens nearly every row."""
    rng = np.random.default_rng(seed)
    return np.repeat(rng.random((n // copies, d), dtype=np.float32), copies, axis=0)


WORKLOADS = {
    # name: (generator, kwargs, min_samples, min_cluster_size)
    "blobs_2k_d10": (blobs_with_noise, dict(n=2000, d=10, seed=42), 5, 5),
    "aniso_100k_d64": (anisotropic_mixture, dict(n=100_000, d=64, seed=43), 10, 50),
    "vmf_500k_d128": (vmf_like, dict(n=500_000, d=128, seed=44), 15, 100),
    # profiling case of the symmetric Borůvka screen (not a benchmark configuration)
    "triplicates_150k_d8": (repeated_points, dict(n=150_000, d=8, seed=3), 5, 5),
}


def workload(name: str, n: int | None = None):
    """(x, min_samples, min_cluster_size) for a named workload, optionally resized to n rows."""
    gen, kw, ms, mcs = WORKLOADS[name]
    kw = dict(kw)
    if n is not None:
        kw["n"] = n
    return gen(**kw), ms, mcs
