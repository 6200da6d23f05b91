"""Batched nested-sampling driver with device-resident live points.

The reference drives its likelihood with MultiNest, one point per callback
(src/retrieval/multinest_loglike.cpp:152-186, Retrieval::doRetrieval
src/retrieval/retrieval.cpp:180-238). Here the live points stay in device memory
as unit-hypercube coordinates and every likelihood call is a batch: candidate
points are drawn on the device, pushed through the device prior transform and
the batched likelihood (``Engine.loglike_cube_batch``), and accepted on the
device.

Algorithm: nested sampling (Skilling 2006, Bayesian Analysis 1, 833) with k live
points replaced per iteration (the k lowest; the j-th of them shrinks the prior
volume by an expected factor (n - j) / (n - j + 1), Henderson et al. 2017,
Stat. Comput. 27, 1287), new points drawn uniformly inside the bounding ellipsoid
of the surviving live points enlarged by ``enlarge`` (Mukherjee, Parkinson &
Liddle 2006, ApJ 638, L51; the single-ellipsoid mode of MultiNest), clipped to
the unit cube, and accepted when their log-likelihood exceeds the current
threshold. The run stops when the live points can add at most ``dlogz`` to
log Z. The evidence error is the usual sqrt(H / n_live).

``loglike`` is any callable taking a (B, ndim) float64 tensor of hypercube points
on ``device`` and returning a (B,) float64 tensor of log-likelihoods (neglected
models return -1e30 and are never accepted).
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable, Optional


@dataclass
class NestedResult:
    log_z: float            # log evidence
    log_z_err: float        # sqrt(information / n_live)
    information: float      # H (nats)
    samples: object         # (S, ndim) tensor: dead points then the final live points (hypercube)
    log_weights: object     # (S,) normalised log posterior weights
    log_l: object           # (S,) log-likelihoods
    n_calls: int            # likelihood evaluations
    n_iter: int


def _logaddexp(a: float, b: float) -> float:
    if a == -math.inf:
        return b
    if b == -math.inf:
        return a
    m = max(a, b)
    return m + math.log1p(math.exp(-abs(a - b)))


def _accumulate(log_z: float, h: float, log_w, log_l):
    """Skilling's running update of log Z and the information H over dead points."""
    for lwj, lj in zip(log_w, log_l):
        log_z_new = _logaddexp(log_z, lwj)
        if log_z_new == -math.inf:
            continue
        prev = math.exp(log_z - log_z_new) * (h + log_z) if log_z > -math.inf else 0.0
        h = math.exp(lwj - log_z_new) * lj + prev - log_z_new
        log_z = log_z_new
    return log_z, h


class BatchedNestedSampler:
    def __init__(self, loglike: Callable, ndim: int, n_live: int = 400, batch: int = 512,
                 replace: Optional[int] = None, enlarge: float = 1.5, dlogz: float = 0.1,
                 max_calls: int = 10_000_000, device: str = "cuda", seed: int = 0):
        import torch
        if n_live < ndim + 2:
            raise ValueError("n_live must exceed ndim + 1 (the ellipsoid needs a full-rank covariance)")
        self.loglike = loglike
        self.ndim = int(ndim)
        self.n_live = int(n_live)
        self.batch = int(batch)
        self.replace = int(replace) if replace else max(1, self.n_live // 10)
        self.enlarge = float(enlarge)
        self.dlogz = float(dlogz)
        self.max_calls = int(max_calls)
        self.device = torch.device(device)
        self.gen = torch.Generator(device=self.device)
        self.gen.manual_seed(int(seed))

    # ------------------------------------------------------------------ proposals
    def _ellipsoid(self, pts):
        """Centre, Cholesky factor of the enlarged bounding ellipsoid of pts."""
        import torch
        c = pts.mean(dim=0)
        d = pts - c
        cov = d.T @ d / max(pts.shape[0] - 1, 1)
        cov = cov + 1e-12 * torch.eye(self.ndim, dtype=pts.dtype, device=pts.device)
        inv = torch.linalg.inv(cov)
        r2 = ((d @ inv) * d).sum(dim=1).max()  # Mahalanobis radius enclosing every point
        cov = cov * (r2 * self.enlarge ** 2)
        return c, torch.linalg.cholesky(cov)

    def _draw(self, c, chol, n):
        """n points uniform in the ellipsoid c + chol * ball, clipped to the unit cube."""
        import torch
        z = torch.randn(n, self.ndim, dtype=torch.float64, device=self.device, generator=self.gen)
        z = z / z.norm(dim=1, keepdim=True)
        r = torch.rand(n, 1, dtype=torch.float64, device=self.device, generator=self.gen) ** (1.0 / self.ndim)
        x = c + (z * r) @ chol.T
        inside = ((x >= 0.0) & (x <= 1.0)).all(dim=1)
        return x[inside]

    # ------------------------------------------------------------------ run
    def run(self) -> NestedResult:
        import torch
        n, k = self.n_live, self.replace
        live = torch.rand(n, self.ndim, dtype=torch.float64, device=self.device, generator=self.gen)
        live_l = self.loglike(live).to(torch.float64)
        calls = n
        dead_x, dead_l, dead_lw = [], [], []
        log_z = -math.inf
        h = 0.0
        log_x = 0.0  # log prior volume enclosed by the current threshold
        it = 0
        while True:
            order = torch.argsort(live_l)
            worst = order[:k]
            lw_l = live_l[worst]
            # the j-th lowest of n shrinks X by (n - j) / (n - j + 1); its weight is the volume between
            steps = torch.arange(k, dtype=torch.float64, device=self.device)
            log_t = torch.log((n - steps) / (n - steps + 1.0))
            log_x_new = log_x + torch.cumsum(log_t, dim=0)
            log_x_prev = torch.cat([torch.tensor([log_x], dtype=torch.float64, device=self.device), log_x_new[:-1]])
            log_dx = log_x_prev + torch.log1p(-torch.exp(log_t))
            lw = lw_l + log_dx
            log_z, h = _accumulate(log_z, h, lw.tolist(), lw_l.tolist())
            dead_x.append(live[worst].clone())
            dead_l.append(lw_l.clone())
            dead_lw.append(lw.clone())
            log_x = float(log_x_new[-1])
            threshold = lw_l[-1]
            it += 1
            # stop when the live points can add at most dlogz
            keep = order[k:]
            max_l = float(live_l[keep].max())
            if max_l + log_x - log_z < math.log(math.expm1(self.dlogz)) or calls >= self.max_calls:
                live = live[keep]
                live_l = live_l[keep]
                break
            # replace the k lowest with points above the threshold
            c, chol = self._ellipsoid(live[keep])
            new_x, new_l = [], []
            got = 0
            empty = 0
            while got < k and calls < self.max_calls:
                x = self._draw(c, chol, self.batch)
                if x.shape[0] == 0:
                    empty += 1
                    if empty > 1000:  # the bound has left the cube: nothing more to draw
                        break
                    continue
                l = self.loglike(x).to(torch.float64)
                calls += x.shape[0]
                ok = l > threshold
                new_x.append(x[ok])
                new_l.append(l[ok])
                got += int(ok.sum())
            if got < k:
                live = live[keep]
                live_l = live_l[keep]
                break
            live = torch.cat([live[keep], torch.cat(new_x)[:k]])
            live_l = torch.cat([live_l[keep], torch.cat(new_l)[:k]])
        # the remaining live points share the last volume equally
        m = live.shape[0]
        lw_live = live_l + (log_x - math.log(m))
        log_z, h = _accumulate(log_z, h, lw_live.tolist(), live_l.tolist())
        samples = torch.cat(dead_x + [live])
        log_l = torch.cat(dead_l + [live_l])
        log_w = torch.cat(dead_lw + [lw_live]) - log_z
        return NestedResult(log_z=log_z, log_z_err=math.sqrt(max(h, 0.0) / n), information=h, samples=samples,
                            log_weights=log_w, log_l=log_l, n_calls=calls, n_iter=it)
