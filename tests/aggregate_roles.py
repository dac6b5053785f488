"""Oracle-backed aggregate roles for the host aggregate driver's tests:
the same interface as cuminlp_gb300.aggregate.DeviceAggregateRoles, with the
oracle's aggregate bound and sampler behind it."""

from __future__ import annotations

import numpy as np

import oracle as O


class OracleAggregateRoles:
    def __init__(self, problem, bound_regions: int, k: int, sample_regions: int, sample_points: int = 1):
        self.op = O.OracleProblem(problem)
        self.n, self.k, self.ns, self.s = bound_regions, k, sample_regions, sample_points

    def n_samples(self) -> int:
        return self.ns * self.s

    def bound_children(self, box, launch):
        flat = np.array([x for b in box for x in b], dtype=np.float64)
        return self.op.aggregate_bound(flat, launch.kinds, launch.var_ids, launch.widths, self.n, self.k, threads=1)

    def sample(self, box, launch, salt):
        flat = np.array([x for b in box for x in b], dtype=np.float64)
        found, value, point, _ = self.op.sample(flat, launch.kinds, launch.var_ids, launch.widths, self.ns, self.s,
                                                salt, threads=1)
        return found, value, point
