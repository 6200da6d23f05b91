"""Joint emission + transmission likelihood.

The reference has no joint model; a joint retrieval is the sum of the
log-likelihoods of two forward models, an emission model and a transmission
model, evaluated on the same spectral grid and sharing their opacity tables:

    log L(theta_e, theta_t) = log L_emission(theta_e) + log L_transmission(theta_t)

Each model is an ordinary engine model. It carries the other model's
observations with likelihood weight 0 (a reference feature: the observation
defines grid points but adds nothing to log L), so both models sample the
identical spectral grid, and the engine then finds the second model's tables
already on the device and shares them (``Engine.table_sharing``).

The joint parameter vector is the emission model's parameters followed by the
transmission model's; tie parameters (e.g. the temperature profile or the
abundances) by writing the same value into both halves and adding the two
gradient halves. A batch row is neglected (log L = -1e30) when either model
neglects it.
"""

from __future__ import annotations

import dataclasses
from typing import List, Sequence, Tuple

import numpy as np

from .config import ObservationArrays
from .retrieval import BatchEvaluator, Engine


def _weightless(o: ObservationArrays) -> ObservationArrays:
    return dataclasses.replace(o, weight=np.zeros(o.n, dtype=np.float64))


def joint_observation_sets(emission: Sequence[ObservationArrays], transmission: Sequence[ObservationArrays]
                           ) -> Tuple[List[ObservationArrays], List[ObservationArrays]]:
    """Observation lists of the two models: each model's own observations
    followed by the other model's with likelihood weight 0."""
    em = list(emission) + [_weightless(o) for o in transmission]
    tr = list(transmission) + [_weightless(o) for o in emission]
    return em, tr


class JointEngine:
    """Emission and transmission engines on one device, one spectral grid and one
    set of device opacity tables."""

    def __init__(self, emission_config: str, emission_obs: Sequence[ObservationArrays], transmission_config: str,
                 transmission_obs: Sequence[ObservationArrays], device: int = 0):
        em, tr = joint_observation_sets(emission_obs, transmission_obs)
        self.emission = Engine(emission_config, em, device=device)
        self.transmission = Engine(transmission_config, tr, device=device)
        if self.emission.N != self.transmission.N:
            raise RuntimeError("the two models did not sample the same spectral grid")
        self.device = int(device)
        self.Pe = self.emission.P
        self.Pt = self.transmission.P
        self.P = self.Pe + self.Pt
        self.N = self.emission.N
        self.n_em_obs = len(emission_obs)
        self.n_tr_obs = len(transmission_obs)

    def tables_shared(self) -> bool:
        return self.transmission.table_sharing()[0]

    def _split(self, params):
        return params[:, :self.Pe].contiguous(), params[:, self.Pe:].contiguous()

    @staticmethod
    def _combine(ll_e, ng_e, ll_t, ng_t):
        import torch
        ng = ng_e | ng_t
        ll = torch.where(ng.bool(), torch.full_like(ll_e, -1e30), ll_e + ll_t)
        return ll, ng

    def loglike_batch(self, params):
        """params: torch float64 CUDA (B, Pe + Pt). Returns (log L (B,), neglect (B,) uint8)."""
        pe, pt = self._split(params)
        ll_e, ng_e = self.emission.loglike_batch(pe)
        ll_t, ng_t = self.transmission.loglike_batch(pt)
        return self._combine(ll_e, ng_e, ll_t, ng_t)

    def grad_batch(self, params):
        """(log L (B,), d log L / d params (B, Pe + Pt), neglect (B,)); neglected rows get zeros."""
        import torch
        pe, pt = self._split(params)
        ll_e, g_e, ng_e = self.emission.grad_batch(pe)
        ll_t, g_t, ng_t = self.transmission.grad_batch(pt)
        ll, ng = self._combine(ll_e, ng_e, ll_t, ng_t)
        g = torch.cat([g_e, g_t], dim=1)
        g[ng.bool()] = 0.0
        return ll, g, ng

    def close(self) -> None:
        self.emission.close()
        self.transmission.close()


class JointBatchEvaluator:
    """Joint log-likelihoods of a fixed-size batch through two captured graphs
    (one per model) on the same stream."""

    def __init__(self, joint: JointEngine, params, autotune: bool = True):
        pe, pt = joint._split(params.detach())
        self.joint = joint
        self.em = BatchEvaluator(joint.emission, pe, autotune=autotune)
        self.tr = BatchEvaluator(joint.transmission, pt, autotune=autotune)

    def __call__(self, params=None):
        if params is not None:
            pe, pt = self.joint._split(params)
            self.em.params.copy_(pe, non_blocking=True)
            self.tr.params.copy_(pt, non_blocking=True)
        ll_e, ng_e = self.em()
        ll_t, ng_t = self.tr()
        return JointEngine._combine(ll_e, ng_e, ll_t, ng_t)

    def close(self) -> None:
        self.em.close()
        self.tr.close()
