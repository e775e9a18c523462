"""Seeded synthetic single-cell workloads for the MWU differential-expression path.

These stand in for real perturbation-screen matrices (none ships with this project). Each
generator returns a CSC matrix as raw arrays (values, int64 row ids, int64 column
pointers) plus an int32 ``group_id`` (0 = reference, 1..T = targets, -1 = ignored), the
layout ``hpdex.backend.mannwhitneyu`` consumes.

Workloads (cells x genes):
  * ``small_float``    2,000 x 500, 4 targets of 250 cells, log1p(Poisson+1) values
  * ``umi_counts``     50,000 x 2,000 integral float32 NB counts, 49 targets
  * ``perturb_screen`` 200,000 x 8,000 log1p-CP10k NB counts, 500 targets
  * ``exact_small``    60,000 x 4,000 dense N(0,1) with per-target shifts, 1,500 targets
                       of 3..40 cells against a 40-cell reference
All draws come from ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Workload:
    name: str
    n_rows: int
    n_cols: int
    data: np.ndarray       # values, CSC order
    indices: np.ndarray    # int64 row ids
    indptr: np.ndarray     # int64 column pointers (n_cols + 1)
    group_id: np.ndarray   # int32 per row
    n_targets: int
    options: dict

    @property
    def nnz(self) -> int:
        return int(self.indptr[-1])

    def csc(self):
        import scipy.sparse as sp
        return sp.csc_matrix((self.data, self.indices, self.indptr), shape=(self.n_rows, self.n_cols))


def _bernoulli_rows(rng, n_rows, density):
    """Sorted row ids of a column whose cells are nonzero with probability `density`."""
    if density <= 0.0:
        return np.zeros(0, np.int64)
    if density >= 1.0:
        return np.arange(n_rows, dtype=np.int64)
    est = int(n_rows * density * 1.3) + 64
    gaps = rng.geometric(density, size=est)
    rows = np.cumsum(gaps) - 1
    while rows[-1] < n_rows - 1:
        more = rng.geometric(density, size=est)
        rows = np.concatenate([rows, rows[-1] + np.cumsum(more)])
    return rows[rows < n_rows].astype(np.int64)


def _nb(rng, mean, r, size):
    """Negative binomial with mean `mean` and size `r` (variance mean + mean^2 / r)."""
    p = r / (r + mean)
    return rng.negative_binomial(r, p, size=size)


def _columns(rng, n_rows, densities, draw):
    """Builds CSC arrays column by column. draw(j, k) returns k values for column j."""
    rows_list, vals_list = [], []
    indptr = np.zeros(len(densities) + 1, np.int64)
    for j, d in enumerate(densities):
        rows = _bernoulli_rows(rng, n_rows, float(d))
        rows_list.append(rows)
        vals_list.append(draw(j, rows.size))
        indptr[j + 1] = indptr[j] + rows.size
    indices = np.concatenate(rows_list) if rows_list else np.zeros(0, np.int64)
    values = np.concatenate(vals_list) if vals_list else np.zeros(0)
    return values, indices, indptr


def _assign_groups(rng, n_rows, ref_size, target_sizes, shuffle=True):
    gid = np.full(n_rows, -1, np.int32)
    order = rng.permutation(n_rows) if shuffle else np.arange(n_rows)
    pos = 0
    gid[order[pos:pos + ref_size]] = 0
    pos += ref_size
    for t, s in enumerate(target_sizes):
        gid[order[pos:pos + s]] = t + 1
        pos += s
    return gid


def small_float(seed: int = 1234, n_rows: int = 2000, n_cols: int = 500) -> Workload:
    """2,000 cells x 500 genes; gene density ~ Beta(1, 9); values log1p(Poisson(l)+1) with
    l ~ Gamma(0.5, scale 4); reference = first half of the cells, 4 equal targets."""
    rng = np.random.default_rng(seed)
    dens = rng.beta(1.0, 9.0, size=n_cols)
    lam = rng.gamma(0.5, 4.0, size=n_cols)
    values, indices, indptr = _columns(
        rng, n_rows, dens, lambda j, k: np.log1p(rng.poisson(lam[j], size=k) + 1.0))
    half = n_rows // 2
    per = (n_rows - half) // 4
    gid = np.full(n_rows, -1, np.int32)
    gid[:half] = 0
    for t in range(4):
        gid[half + t * per: half + (t + 1) * per] = t + 1
    return Workload("small_float", n_rows, n_cols, values.astype(np.float32), indices, indptr, gid, 4,
                    dict(tie_correction=True, use_continuity=True, zero_handling="min"))


def _scaled_sizes(sizes, room, floor_min):
    sizes = np.floor(sizes * (room / sizes.sum())).astype(np.int64)
    return np.maximum(sizes, floor_min)


def umi_counts(seed: int = 2024, n_rows: int = 50_000, n_cols: int = 2_000,
               mu_log_loc: float = -1.0, n_targets: int = 49) -> Workload:
    """Integral float32 UMI counts: c ~ NB(mean mu_g, size 2) with mu_g ~ LogNormal(loc, 1.5)
    clipped to [0.01, 50]; reference 10,000 cells; target sizes ~ LogNormal(ln 400, 0.8)
    clipped to [100, 2000] and scaled so that 98 % of cells are assigned (2 % ignored)."""
    rng = np.random.default_rng(seed)
    mu = np.clip(rng.lognormal(mu_log_loc, 1.5, size=n_cols), 0.01, 50.0)
    # a cell is stored iff its count is nonzero: draw per-gene nonzero probability exactly
    p_zero = (2.0 / (2.0 + mu)) ** 2.0
    dens = 1.0 - p_zero

    def draw(j, k):
        # counts conditioned on being nonzero (rejection from the NB)
        out = np.empty(k, np.int64)
        filled = 0
        while filled < k:
            c = _nb(rng, mu[j], 2.0, size=max(2 * (k - filled), 16))
            c = c[c > 0][: k - filled]
            out[filled:filled + c.size] = c
            filled += c.size
        return out.astype(np.float32)

    values, indices, indptr = _columns(rng, n_rows, dens, draw)
    ref = n_rows // 5
    sizes = np.clip(rng.lognormal(np.log(400.0), 0.8, size=n_targets), 100, 2000)
    sizes = _scaled_sizes(sizes, int(0.98 * n_rows) - ref, 2)
    gid = _assign_groups(rng, n_rows, ref, sizes)
    return Workload("umi_counts", n_rows, n_cols, values.astype(np.float32), indices, indptr, gid,
                    n_targets, dict(tie_correction=True, use_continuity=True, zero_handling="min"))


def perturb_screen(seed: int = 7, n_rows: int = 200_000, n_cols: int = 8_000,
                   n_targets: int = 500, ref_size: int = 20_000) -> Workload:
    """log1p-CP10k float32 at perturbation-screen scale: gene density ~ Beta(0.5, 5); stored
    counts 1 + NB(size 2, mean mu_g), mu_g ~ LogNormal(-1, 1.5) clipped to [0.01, 50]; each
    cell divided by its library size, x 1e4, log1p. Reference 20,000 cells; 500 targets of
    LogNormal(ln 300, 1.0) clipped to [20, 3000], scaled to fit the remaining cells (floor,
    at least 20); the rest are ignored (-1)."""
    rng = np.random.default_rng(seed)
    dens = rng.beta(0.5, 5.0, size=n_cols)
    mu = np.clip(rng.lognormal(-1.0, 1.5, size=n_cols), 0.01, 50.0)
    counts, indices, indptr = _columns(
        rng, n_rows, dens, lambda j, k: 1 + _nb(rng, mu[j], 2.0, size=k))
    lib = np.bincount(indices, weights=counts, minlength=n_rows)
    lib[lib == 0] = 1.0
    values = np.log1p(counts / lib[indices] * 1e4).astype(np.float32)
    sizes = np.clip(rng.lognormal(np.log(300.0), 1.0, size=n_targets), 20, 3000)
    sizes = _scaled_sizes(sizes, n_rows - ref_size, 20)
    while ref_size + sizes.sum() > n_rows:  # clamping at 20 can overshoot: trim the largest
        sizes[np.argmax(sizes)] -= ref_size + sizes.sum() - n_rows
    gid = _assign_groups(rng, n_rows, ref_size, sizes)
    return Workload("perturb_screen", n_rows, n_cols, values, indices, indptr, gid, n_targets,
                    dict(tie_correction=True, use_continuity=True, zero_handling="min"))


def exact_small(seed: int = 11, n_rows: int = 60_000, n_cols: int = 4_000, n_targets: int = 1500,
                ref_size: int = 40) -> Workload:
    """Dense N(0,1) float32 stored as CSC (every cell explicit); each target adds a shift
    delta ~ N(0, 0.3^2) per gene to its cells. Reference 40 cells, targets of U{3..40}
    cells; the remaining cells are ignored. Intended for method='exact'."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(3, 41, size=n_targets)
    gid = _assign_groups(rng, n_rows, ref_size, sizes)
    shift = rng.normal(0.0, 0.3, size=(n_targets + 1, n_cols)).astype(np.float32)
    shift[0] = 0.0
    X = rng.standard_normal((n_cols, n_rows), dtype=np.float32)  # gene-major == CSC order
    g = np.where(gid > 0, gid, 0)
    for c0 in range(0, n_cols, 256):  # add the per-(target, gene) shift in column blocks
        X[c0:c0 + 256] += shift[g, c0:c0 + 256].T
    indptr = np.arange(n_cols + 1, dtype=np.int64) * n_rows
    indices = np.tile(np.arange(n_rows, dtype=np.int64), n_cols)
    return Workload("exact_small", n_rows, n_cols, X.reshape(-1), indices, indptr, gid, n_targets,
                    dict(tie_correction=True, use_continuity=False, zero_handling="none",
                         method="exact"))


def extreme_shift(seed: int = 31, n_cols: int = 400) -> Workload:
    """Strong differential signal, for the deep tail of the p-values: 20,000 reference cells
    and targets of 3,000, 1,000 and 3,000 cells (27,000 cells, all assigned). Values are
    quantised sums of four uniform integers in [0, 63], / 16 (Irwin-Hall, sd ~2.3 units, so
    ties occur); each target adds its own per-gene shift in sd units: target 1 U[0.6, 1.0]
    (|z| near 30-48, around the p-values' subnormal range), target 2 U[1.2, 1.8], target 3
    U[0, 1.6]. 70 % of the genes are dense, the rest keep each cell with probability U[0.5, 1)
    (implicit zeros join the zero block). Only integer draws are used, so the arrays are
    bit-identical on every platform and numpy version (the stored reference outputs depend on
    that)."""
    rng = np.random.default_rng(seed)
    ref, sizes = 20_000, np.array([3_000, 1_000, 3_000])
    n_rows = ref + int(sizes.sum())
    gid = np.zeros(n_rows, np.int32)
    pos = ref
    for t, s in enumerate(sizes):
        gid[pos:pos + s] = t + 1
        pos += s
    perm = rng.permutation(n_rows)  # integer-based shuffle
    gid = gid[perm]
    sd_units = 16.0 * np.sqrt(4 * (64 * 64 - 1) / 12.0) / 16.0  # sd of the integer sum, in 1/16
    lo = np.array([0, 600, 1200, 0])  # shifts in thousandths of an sd, per target
    hi = np.array([0, 1000, 1800, 1600])
    rows_list, vals_list = [], []
    indptr = np.zeros(n_cols + 1, np.int64)
    for j in range(n_cols):
        shift_milli = np.array([0] + [int(rng.integers(lo[t], hi[t] + 1)) for t in (1, 2, 3)])
        # shift in 1/16 units, rounded to an integer so values stay exact in float32
        shift16 = np.round(shift_milli * sd_units / 1000.0).astype(np.int64)
        base = rng.integers(0, 64, size=(4, n_rows)).sum(axis=0)
        v = base + shift16[gid]
        if rng.integers(0, 10) < 7:
            rows = np.arange(n_rows, dtype=np.int64)
        else:
            keep_milli = int(rng.integers(500, 1000))
            rows = np.nonzero(rng.integers(0, 1000, size=n_rows) < keep_milli)[0].astype(np.int64)
        rows_list.append(rows)
        vals_list.append((v[rows] / 16.0).astype(np.float32))
        indptr[j + 1] = indptr[j] + rows.size
    return Workload("extreme_shift", n_rows, n_cols, np.concatenate(vals_list),
                    np.concatenate(rows_list), indptr, gid, 3,
                    dict(tie_correction=True, use_continuity=True, zero_handling="min"))


WORKLOADS = {
    "small_float": small_float,
    "umi_counts": umi_counts,
    "perturb_screen": perturb_screen,
    "exact_small": exact_small,
}


def resident_atlas(seed: int = 13, n_rows: int = 1_000_000, n_cols: int = 20_000,
                   per_col: int = 50_000):
    """The serving workload's largest matrix, generated on the GPU (host generation of 1e9
    entries would take minutes) and made resident: (log1p-CP10k float32 matrix, integer-count
    twin), both ResidentMatrix. Every gene stores per_col cells (5 % density at the defaults):
    row i*s + jitter, s = n_rows // per_col, jitter uniform in [0, s), so rows ascend and never
    repeat. Counts are 1 + NB(size 2, mean mu_g), mu_g ~ LogNormal(-1, 1.5) clipped to [0.01, 50]
    (a gamma-Poisson mixture); the float matrix holds log1p(count / library size * 1e4) of each
    cell, the twin the counts themselves. torch does the generation (device memory plumbing)."""
    import torch
    from .resident import ResidentMatrix
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(seed)
    stride = n_rows // per_col
    rows = (torch.arange(per_col, device=dev, dtype=torch.int32) * stride)[None, :] + \
        torch.randint(0, stride, (n_cols, per_col), device=dev, generator=g, dtype=torch.int32)
    rows = rows.reshape(-1)
    mu = torch.exp(torch.randn(n_cols, device=dev, generator=g) * 1.5 - 1.0).clamp_(0.01, 50.0)
    shape = torch.full((n_cols, per_col), 2.0, device=dev)
    lam = torch._standard_gamma(shape, generator=g) * (mu[:, None] / 2.0)
    del shape
    counts = (torch.poisson(lam, generator=g) + 1.0).reshape(-1)
    del lam
    lib = torch.zeros(n_rows, device=dev, dtype=torch.float32).index_add_(0, rows.long(), counts)
    lib.clamp_(min=1.0)
    values = torch.log1p(counts * (1e4 / lib[rows.long()]))
    torch.cuda.synchronize()
    indptr = np.arange(n_cols + 1, dtype=np.int64) * per_col
    M = ResidentMatrix.from_device(values.data_ptr(), rows.data_ptr(), indptr, n_rows, np.float32)
    Mi = ResidentMatrix.from_device(counts.data_ptr(), rows.data_ptr(), indptr, n_rows, np.float32)
    del values, counts, rows, lib
    torch.cuda.empty_cache()
    return M, Mi
