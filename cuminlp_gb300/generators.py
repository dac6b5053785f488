"""Seeded synthetic (MI)QCQP instances of the benchmark shapes.

Every instance is built through the Problem/Expr API the way a modeller
writes x^T Q x + c^T x with the reference's builder: for each upper-
triangle pair (i <= j) in row-major order one term ``coef * (x_i * x_j)``
(``x_i * x_i`` emits Sqr), accumulated left to right, then the linear
terms ``c_i * x_i``.  Constraints follow the same pattern with their own
matrices.

Random numbers come from a SplitMix64 stream; a standard normal draw is
the Irwin-Hall sum of twelve uniforms minus six (mean 0, variance 1).
Both use integer and IEEE add/multiply only, so an instance is bit-for-bit
the same on every host.  Seeds: 0xC0FFEE ^ (family << 32) ^ instance, where
the family number is fixed per generator below (1: n=4 QCQP, 2: n=32
MIQCQP, 3: n=64 MIQCQP, 4: uneven batch instances, 5: serving requests).
"""

from __future__ import annotations

from dataclasses import dataclass

from . import _abi as A
from .problem import Expr, Problem

MASK64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self) -> float:
        """U[0, 1) with 53 random bits."""
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)

    def uniform_range(self, a: float, b: float) -> float:
        return a + (b - a) * self.uniform()

    def normal(self) -> float:
        s = 0.0
        for _ in range(12):
            s += self.uniform()
        return s - 6.0

    def integer(self, lo: int, hi: int) -> int:
        """Uniform integer in [lo, hi]."""
        return lo + self.next() % (hi - lo + 1)


def seed_for(family: int, instance: int = 0) -> int:
    return 0xC0FFEE ^ (family << 32) ^ instance


@dataclass
class QCQPSpec:
    n: int
    m: int
    n_int: int = 0
    int_lb: float = 0.0
    int_ub: float = 7.0
    cont_lb: float = -10.0
    cont_ub: float = 10.0
    q_density: float = 1.0
    a_density: float = 1.0
    rhs: tuple = (5.0, 5.0)  # constant or (lo, hi) for U[lo, hi]
    linear: bool = True


def _sym_terms(rng: SplitMix64, n: int, density: float):
    """Upper-triangle entries (i, j, q) of a symmetric N(0,1) matrix with a
    Bernoulli(density) mask, row-major."""
    out = []
    for i in range(n):
        for j in range(i, n):
            keep = density >= 1.0 or rng.uniform() < density
            q = rng.normal()
            if keep:
                out.append((i, j, q))
    return out


def _quadratic(x: list[Expr], terms, lin) -> Expr:
    acc = None
    for i, j, q in terms:
        coef = q if i == j else 2.0 * q
        t = coef * (x[i] * x[j])
        acc = t if acc is None else acc + t
    for i, c in enumerate(lin):
        t = c * x[i]
        acc = t if acc is None else acc + t
    return acc


def qcqp(spec: QCQPSpec, seed: int) -> Problem:
    rng = SplitMix64(seed)
    p = Problem()
    x = []
    for v in range(spec.n):
        if v < spec.n_int:
            x.append(p.int_var(spec.int_lb, spec.int_ub))
        else:
            x.append(p.var(spec.cont_lb, spec.cont_ub))
    q_terms = _sym_terms(rng, spec.n, spec.q_density)
    c = [rng.normal() for _ in range(spec.n)] if spec.linear else []
    p.set_objective(_quadratic(x, q_terms, c))
    for _ in range(spec.m):
        a_terms = _sym_terms(rng, spec.n, spec.a_density)
        b = [rng.normal() for _ in range(spec.n)] if spec.linear else []
        lo, hi = spec.rhs
        r = lo if lo == hi else rng.uniform_range(lo, hi)
        if not a_terms and not b:
            continue
        p.add_constraint(_quadratic(x, a_terms, b), A.CMP_LE, r)
    return p


# ---- the benchmark workloads ------------------------------------------
def qcqp_n4(instance: int = 0) -> Problem:
    """n=4 continuous in [-10,10]; Q, A dense symmetric N(0,1); c, b N(0,1);
    one constraint x^T A x + b^T x <= 5."""
    return qcqp(QCQPSpec(n=4, m=1, cont_lb=-10, cont_ub=10, rhs=(5.0, 5.0)), seed_for(1, instance))


def miqcqp_n32(instance: int = 0) -> Problem:
    """n=32: 4 integers in [0,7] + 28 continuous in [-5,5]; Q dense; m=16
    constraints with A_i at 20% density, b_i N(0,1), r_i U[1,10]."""
    return qcqp(QCQPSpec(n=32, m=16, n_int=4, int_lb=0, int_ub=7, cont_lb=-5, cont_ub=5, q_density=1.0,
                         a_density=0.2, rhs=(1.0, 10.0)), seed_for(2, instance))


def miqcqp_n64(instance: int = 0) -> Problem:
    """n=64: 8 integers in [0,15] + 56 continuous in [-10,10]; Q at 30%
    density; m=32 constraints at 10% density."""
    return qcqp(QCQPSpec(n=64, m=32, n_int=8, int_lb=0, int_ub=15, cont_lb=-10, cont_ub=10, q_density=0.3,
                         a_density=0.1, rhs=(1.0, 10.0)), seed_for(3, instance))


def uneven_qcqp(instance: int) -> Problem:
    """One of the 1024 uneven instances: n ~ U{4..48}, m ~ U{0..24},
    integer share U[0, 0.25], densities U[0.1, 1.0], bounds [-10, 10]."""
    rng = SplitMix64(seed_for(4, instance) ^ 0x5A5A5A5A)
    n = rng.integer(4, 48)
    m = rng.integer(0, 24)
    n_int = int(rng.uniform_range(0.0, 0.25) * n)
    qd = rng.uniform_range(0.1, 1.0)
    ad = rng.uniform_range(0.1, 1.0)
    return qcqp(QCQPSpec(n=n, m=m, n_int=n_int, int_lb=-10, int_ub=10, cont_lb=-10, cont_ub=10, q_density=qd,
                         a_density=ad, rhs=(1.0, 10.0)), seed_for(4, instance))


def serving_qcqp(instance: int) -> Problem:
    """A serving request: n in {8,16,32,64} with weights 0.4/0.3/0.2/0.1,
    m = n/2, 10% integers, densities U[0.1, 1.0]."""
    rng = SplitMix64(seed_for(5, instance) ^ 0xA5A5A5A5)
    u = rng.uniform()
    n = 8 if u < 0.4 else 16 if u < 0.7 else 32 if u < 0.9 else 64
    qd = rng.uniform_range(0.1, 1.0)
    ad = rng.uniform_range(0.1, 1.0)
    return qcqp(QCQPSpec(n=n, m=n // 2, n_int=n // 10, int_lb=-10, int_ub=10, cont_lb=-10, cont_ub=10,
                         q_density=qd, a_density=ad, rhs=(1.0, 10.0)), seed_for(5, instance))


# the three single-problem workloads, keyed by their variable count
BY_N = {4: qcqp_n4, 32: miqcqp_n32, 64: miqcqp_n64}
