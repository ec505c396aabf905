"""The learned surrogate and the parameter sweeps it screens.

`Surrogate` wraps one handle of include/epi_surrogate.h -- an ensemble of `members` MLPs of
one shape, trained and evaluated together by the sm_103a kernels (there is no CPU path).
The rest is host orchestration:

* `PARAMS`: the eight sweep parameters and their ranges (regular and high transmission rate,
  death rate, lockdown threshold, essential-worker fraction, vaccination hour and fraction,
  initial infections), mapped onto engine configs by `config_for`.
* `latin_hypercube` / `uniform_candidates`: designs over the unit cube.
* `simulate_curves`: runs many configs as batched ensembles on the GPU engine and returns
  daily S/E/I/H/R/D at hours 24 d (d = 1..days), normalised by population -- the training
  targets and the sweep's judge.
* `screen`: scores candidates with a surrogate ensemble against a target curve, keeps the
  best, and flags those whose members disagree on the peak by more than a tolerance.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import EpiError, MlpConfig, lib
from .engine import Ensemble
from .workloads import SMALL_POX, config_dict, params_of

COMPARTMENTS = ("susceptible", "exposed", "infected", "hospitalized", "recovered", "deceased")


@dataclass(frozen=True)
class SweepParam:
    name: str
    lo: float
    hi: float
    integer: bool = False


PARAMS = (
    SweepParam("regular_transmission_rate", 0.02, 0.10),
    SweepParam("high_transmission_rate", 0.2, 0.8),
    SweepParam("death_rate", 0.05, 0.3),
    SweepParam("lockdown_at_number_of_infections", 100, 5000, True),
    SweepParam("essential_workers_population", 0.05, 0.3),
    SweepParam("vaccination_hour", 500, 2400, True),
    SweepParam("vaccination_percent", 0.0, 0.4),
    SweepParam("initial_infected", 5, 200, True),
)


def denormalise(u: np.ndarray) -> list[dict]:
    """Unit-cube rows -> parameter dicts (integers rounded)."""
    out = []
    for row in np.atleast_2d(u):
        d = {}
        for p, x in zip(PARAMS, row):
            v = p.lo + float(x) * (p.hi - p.lo)
            d[p.name] = int(round(v)) if p.integer else v
        out.append(d)
    return out


def latin_hypercube(n: int, dims: int, seed: int) -> np.ndarray:
    """n points, one in each of n equal strata of every axis (McKay, Beckman & Conover 1979)."""
    rng = np.random.default_rng(seed)
    u = (np.arange(n)[:, None] + rng.random((n, dims))) / n
    for j in range(dims):
        u[:, j] = u[rng.permutation(n), j]
    return u


def uniform_candidates(n: int, dims: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).random((n, dims))


def config_for(p: dict, agents: int, grid: int, hours: int, seed: int, per_agents: int | None = None) -> dict:
    """Engine config of one parameter point.  The two head counts (initial infections and the
    lockdown threshold) are per `per_agents` agents and scale with the population, so that
    normalised curves of worlds of different sizes are comparable; per_agents=None keeps them
    as absolute counts."""
    scale = 1.0 if per_agents is None else agents / per_agents
    disease = dict(SMALL_POX)
    disease["regular_transmission_rate"] = p["regular_transmission_rate"]
    disease["high_transmission_rate"] = p["high_transmission_rate"]
    disease["death_rate"] = p["death_rate"]
    interventions = [
        {"Lockdown": {"at_number_of_infections": max(1, int(round(p["lockdown_at_number_of_infections"] * scale))),
                      "essential_workers_population": p["essential_workers_population"]}},
        {"Vaccinate": {"at_hour": int(p["vaccination_hour"]), "percent": p["vaccination_percent"]}},
    ]
    exposed = max(1, int(round(p["initial_infected"] * scale)))
    return config_dict(agents, grid, hours, seed, disease, exposed=exposed, interventions=interventions)


def curves_from_rows(rows: np.ndarray, n: int, days: int) -> np.ndarray:
    """Daily compartments (6 x days, compartment-major) at hours 24 d, normalised by n; a run
    that stopped early keeps its last counts."""
    out = np.zeros((6, days))
    hours = rows["hour"].astype(np.int64) if len(rows) else np.zeros(0, dtype=np.int64)
    for d in range(1, days + 1):
        k = np.searchsorted(hours, 24 * d, side="right") - 1
        if k < 0:
            continue
        for c, name in enumerate(COMPARTMENTS):
            out[c, d - 1] = rows[name][k] / n
    return out


def simulate_curves(configs: list[dict], days: int, batch: int = 512) -> np.ndarray:
    """Run configs on the GPU engine in ensembles of `batch`; returns (len, 6 * days)."""
    out = np.zeros((len(configs), 6 * days), dtype=np.float32)
    for s in range(0, len(configs), batch):
        chunk = configs[s:s + batch]
        ens = Ensemble([params_of(c) for c in chunk])
        try:
            rows = ens.run()
        finally:
            ens.close()
        for i, (c, r) in enumerate(zip(chunk, rows)):
            n = c["population"]["Auto"]["number_of_agents"]
            out[s + i] = curves_from_rows(r, n, days).ravel()
    return out


def compartment_scaling(y: np.ndarray, days: int, floor: float = 1e-6):
    """Output standardisation of (n, 6 * days) curves: the mean of every output and one scale
    per compartment (its standard deviation over samples and days), so that the small
    compartments weigh as much in the loss as the large ones."""
    y = np.asarray(y, dtype=np.float64)
    mean = y.mean(axis=0)
    sd = (y - mean).reshape(len(y), 6, days).std(axis=(0, 2))
    return mean, np.repeat(np.maximum(sd, floor), days)


def peak_height(curves: np.ndarray, days: int) -> np.ndarray:
    """Peak of the infected compartment of (n, 6 * days) curves."""
    return np.asarray(curves).reshape(-1, 6, days)[:, 2, :].max(axis=1)


class Surrogate:
    """`members` MLPs on the GPU (epi_mlp_*): in_dim -> hidden x hidden_layers (GELU) -> out_dim.
    Member m is initialised from seed + m and trained on minibatches shuffled from
    train(seed=s) + m: it equals a one-member Surrogate built and trained with those seeds.
    predict() and score() give the ensemble mean; the *_members variants every member's."""

    def __init__(self, in_dim: int = 8, out_dim: int = 600, hidden: int = 512, hidden_layers: int = 3,
                 batch: int = 256, lr: float = 1e-3, seed: int = 0, beta1: float = 0.9, beta2: float = 0.999,
                 eps: float = 1e-8, members: int = 1):
        self.members = int(members)
        self.cfg = MlpConfig(in_dim, hidden, hidden_layers, out_dim, batch, lr, beta1, beta2, eps, self.members, seed)
        h = C.c_void_p()
        rc = lib().epi_mlp_create(C.byref(self.cfg), C.byref(h))
        if rc != _lib.EPI_OK:
            msg = lib().epi_mlp_last_error(h).decode() if h.value else "invalid configuration"
            if h.value:
                lib().epi_mlp_destroy(h)
            raise EpiError(rc, msg)
        self._h = h
        n = C.c_uint64(0)
        self._check(lib().epi_mlp_param_count(self._h, C.byref(n)))
        self.n_params = n.value
        self.shapes = [(hidden, in_dim)] + [(hidden, hidden)] * (hidden_layers - 1) + [(out_dim, hidden)]

    def _check(self, rc):
        if rc != _lib.EPI_OK:
            raise EpiError(rc, lib().epi_mlp_last_error(self._h).decode())

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().epi_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _f32(a) -> np.ndarray:
        return np.ascontiguousarray(a, dtype=np.float32)

    @staticmethod
    def _ptr(a: np.ndarray):
        return a.ctypes.data_as(C.POINTER(C.c_float))

    def _shape(self, a: np.ndarray) -> np.ndarray:
        """(members, ...) -> (...) for a one-member handle."""
        return a[0] if self.members == 1 else a

    def get_params(self) -> np.ndarray:
        """(n_params,) for one member, else (members, n_params)."""
        out = np.zeros((self.members, self.n_params), dtype=np.float32)
        self._check(lib().epi_mlp_get_params(self._h, self._ptr(out)))
        return self._shape(out)

    def set_params(self, flat) -> None:
        a = self._f32(flat)
        assert a.size == self.members * self.n_params
        self._check(lib().epi_mlp_set_params(self._h, self._ptr(a)))

    def set_output_scaling(self, mean, scale) -> None:
        """Train and predict in standardised outputs z = (y - mean) / scale (host side);
        predict() and score() take and return y."""
        self.y_mean = np.asarray(mean, dtype=np.float64).ravel()
        self.y_scale = np.asarray(scale, dtype=np.float64).ravel()
        assert self.y_mean.size == self.cfg.out_dim and self.y_scale.size == self.cfg.out_dim
        assert (self.y_scale > 0).all()

    def _to_z(self, y) -> np.ndarray:
        if getattr(self, "y_mean", None) is None:
            return self._f32(y)
        return self._f32((np.asarray(y, dtype=np.float64) - self.y_mean) / self.y_scale)

    def _from_z(self, z) -> np.ndarray:
        if getattr(self, "y_mean", None) is None:
            return z
        return (z * self.y_scale + self.y_mean).astype(np.float32)

    def set_dataset(self, x, y) -> None:
        x, y = self._f32(x), self._to_z(y)
        assert x.shape[0] == y.shape[0] and x.shape[1] == self.cfg.in_dim and y.shape[1] == self.cfg.out_dim
        self._check(lib().epi_mlp_set_dataset(self._h, self._ptr(x), self._ptr(y), x.shape[0]))

    def train(self, steps: int, seed: int = 0) -> np.ndarray:
        """Per-step losses: (steps,) for one member, else (members, steps)."""
        losses = np.zeros((self.members, max(steps, 1)), dtype=np.float32)
        self._check(lib().epi_mlp_train(self._h, steps, seed, self._ptr(losses)))
        return self._shape(losses[:, :steps])

    def gradients(self, x, y):
        """Loss and gradients of one minibatch: (float, (n_params,)) for one member, else
        ((members,), (members, n_params))."""
        x, y = self._f32(x), self._f32(y)
        g = np.zeros((self.members, self.n_params), dtype=np.float32)
        loss = np.zeros(self.members, dtype=np.float32)
        self._check(lib().epi_mlp_gradients(self._h, self._ptr(x), self._ptr(y), x.shape[0], self._ptr(g),
                                            self._ptr(loss)))
        return (float(loss[0]), g[0]) if self.members == 1 else (loss, g)

    def predict_members(self, x) -> np.ndarray:
        """Every member's curves: (members, n, out_dim)."""
        x = self._f32(x)
        y = np.zeros((self.members, x.shape[0], self.cfg.out_dim), dtype=np.float32)
        self._check(lib().epi_mlp_predict(self._h, self._ptr(x), x.shape[0], self._ptr(y)))
        return self._from_z(y)

    def predict(self, x) -> np.ndarray:
        """The ensemble-mean curves (n, out_dim)."""
        y = self.predict_members(x)
        return y[0] if self.members == 1 else y.mean(axis=0, dtype=np.float64).astype(np.float32)

    def score_members(self, x, target) -> np.ndarray:
        """Squared distance of every member's curves to the target, summed over outputs, in the
        training scale (the standardised outputs when set_output_scaling was called):
        (members, n)."""
        x, t = self._f32(x), self._to_z(np.asarray(target)[None])[0]
        s = np.zeros((self.members, x.shape[0]), dtype=np.float32)
        self._check(lib().epi_mlp_score(self._h, self._ptr(x), x.shape[0], self._ptr(t), self._ptr(s)))
        return s

    def score(self, x, target) -> np.ndarray:
        """The members' mean score_members (n,)."""
        s = self.score_members(x, target)
        return s[0] if self.members == 1 else s.mean(axis=0)

    def kernels_launched(self) -> int:
        v = C.c_uint64(0)
        self._check(lib().epi_mlp_kernels_launched(self._h, C.byref(v)))
        return v.value


def screen(nets, candidates: np.ndarray, target: np.ndarray, keep: int, days: int, peak_tolerance: float = 0.05):
    """Rank candidates by the ensemble-mean squared distance of their predicted curves to the
    target; return (indices of the best `keep`, their mean scores, a mask of those whose
    members' predicted peaks spread by more than peak_tolerance of the mean peak).  nets: a
    Surrogate (all its members) or a list of them."""
    nets = [nets] if isinstance(nets, Surrogate) else list(nets)
    scores = np.concatenate([n.score_members(candidates, target) for n in nets]).mean(axis=0)
    best = np.argsort(scores, kind="stable")[:keep]
    preds = np.concatenate([n.predict_members(candidates[best]) for n in nets])
    peaks = np.stack([peak_height(p, days) for p in preds])
    mean_peak = np.maximum(np.abs(peaks.mean(axis=0)), 1e-12)
    flagged = (peaks.max(axis=0) - peaks.min(axis=0)) / mean_peak > peak_tolerance
    return best, scores[best], flagged


def member_peak_spread(nets, points: np.ndarray, days: int) -> np.ndarray:
    """(max - min) / |mean| of the members' predicted infected peaks at each point."""
    nets = [nets] if isinstance(nets, Surrogate) else list(nets)
    if len(points) == 0:
        return np.zeros(0)
    preds = np.concatenate([n.predict_members(points) for n in nets])
    peaks = np.stack([peak_height(p, days) for p in preds])
    return (peaks.max(axis=0) - peaks.min(axis=0)) / np.maximum(np.abs(peaks.mean(axis=0)), 1e-12)


def screen_with_fallback(nets, candidates: np.ndarray, target: np.ndarray, keep: int, days: int,
                         peak_tolerance: float = 0.05, max_fallback: int | None = None):
    """The surrogate screen with the ABM as its fallback.  Candidates are ranked by the members'
    mean score and the best `keep` are kept.  Where the members disagree the mean cannot be
    trusted, so a candidate outside the kept set is handed to the ABM when (a) at least one
    member scores it within the kept set's worst mean score -- its rank depends on which
    member is believed -- and (b) the members' predicted infected peaks spread by more than
    peak_tolerance of their mean.  Those are taken most promising first (lowest member score),
    at most max_fallback of them (default keep // 4).

    Returns a dict: kept (indices), kept_scores, kept_flagged (mask over kept: members disagree
    by more than peak_tolerance -- re-run by the ABM anyway), fallback (indices for the ABM),
    uncertain (how many candidates met (a)), fallback_eligible (how many met (a) and (b))."""
    nets = [nets] if isinstance(nets, Surrogate) else list(nets)
    member_scores = np.concatenate([n.score_members(candidates, target) for n in nets])
    mean_scores = member_scores.mean(axis=0)
    order = np.argsort(mean_scores, kind="stable")
    kept = order[:keep]
    cut = mean_scores[kept[-1]] if len(kept) else -np.inf
    outside = order[keep:]
    best_member = member_scores[:, outside].min(axis=0)
    uncertain = outside[best_member <= cut]
    uncertain = uncertain[np.argsort(member_scores[:, uncertain].min(axis=0), kind="stable")]
    spread_u = member_peak_spread(nets, candidates[uncertain], days)
    eligible = uncertain[spread_u > peak_tolerance]
    cap = keep // 4 if max_fallback is None else max_fallback
    return {"kept": kept, "kept_scores": mean_scores[kept],
            "kept_flagged": member_peak_spread(nets, candidates[kept], days) > peak_tolerance,
            "fallback": eligible[:cap], "uncertain": int(len(uncertain)), "fallback_eligible": int(len(eligible))}


def relative_peak_error(curves: np.ndarray, reference: np.ndarray, days: int) -> np.ndarray:
    p, q = peak_height(curves, days), peak_height(reference, days)
    return np.abs(p - q) / np.maximum(q, 1e-12)


def unit_distance(u: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Euclidean distance in the unit cube, divided by sqrt(dims) (0 = same point, 1 = opposite corners)."""
    u, v = np.atleast_2d(u), np.atleast_2d(v)
    return np.sqrt(((u - v) ** 2).sum(axis=1)) / math.sqrt(u.shape[1])
