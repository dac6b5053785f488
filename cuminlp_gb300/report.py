"""The reference's machine-read output lines, from an outcome dict.

``tools/minlp_status.py`` in the reference scrapes three things from a
solver's stdout: the ``PARAMS`` line before the search
(source/gams/solve.cu:785-825), ConsoleReporter's finish block with its
``Stop reason:`` and ``Outcome:`` lines (report/observer.hpp:243-284), and
the final tab-separated ``RESULT`` line (source/gams/solve.cu:839-870).
These functions print the same grammar for this solver's outcomes, so the
same tooling reads either.  ``balances`` is RunTelemetry's counter
self-check (report/telemetry.hpp:57-75).
"""

from __future__ import annotations

DBL_MAX = 1.7976931348623157e308


def _g17(x: float) -> str:
    # std::cout with precision(17) in the default float field
    return "%.17g" % x


def _g6(x: float) -> str:
    # std::cout's default precision (6) in the default float field
    return "%g" % x


def params_line(bisection_budget: int, sample_points: int, policy: str = "bisection_budget",
                source: str = "named") -> str:
    """The PARAMS line of a BisectionBudget search."""
    return (f"PARAMS\tpolicy={policy}\tsource={source}\tbisection_budget={int(bisection_budget)}"
            f"\tsample_points={int(sample_points)}")


def result_line(outcome: dict, maximise: bool = False) -> str:
    """RESULT<TAB>sense=min|max<TAB>primal=<value|none><TAB>dual=<value|none>.

    The solver minimises; a maximisation was negated on the way in, so both
    bounds are negated back and keep their roles (primal = incumbent)."""
    ub, lb = outcome["upper_bound"], outcome["lower_bound"]
    found_incumbent = ub < DBL_MAX
    found_dual = lb > -DBL_MAX
    primal = -ub if maximise else ub
    dual = -lb if maximise else lb
    return ("RESULT\tsense=" + ("max" if maximise else "min") + "\tprimal="
            + (_g17(primal) if found_incumbent else "none") + "\tdual=" + (_g17(dual) if found_dual else "none"))


def finish_block(outcome: dict, iter_limit: int | None = None) -> list[str]:
    """ConsoleReporter::on_finish's lines for this outcome."""
    lines = []
    if outcome.get("infeasible"):
        lines.append("Search space exhausted: every region was proven to hold no feasible point, so the problem is "
                     "infeasible as far as interval analysis can tell. Sampling that merely never landed on a "
                     "feasible point would have left regions pending here instead.")
    lines.append("------------ Finished ------------")
    lines.append(f"{_g6(outcome['lower_bound'])} <= min <= {_g6(outcome['upper_bound'])}")
    if outcome.get("proven_optimal"):
        at_limit = iter_limit is not None and outcome["counters"]["expansions"] >= iter_limit
        lines.append("Proven optimal: no pending region can beat the incumbent"
                     + (" (the iteration limit was reached, but every remaining region is already dominated)"
                        if at_limit else "") + ".")
    lines.append("Stop reason: " + outcome["stop_reason"])
    if not outcome["upper_bound"] < DBL_MAX:
        lines.append("Outcome: " + ("infeasible" if outcome.get("infeasible") else "no sample"))
    c = outcome["counters"]
    lines.append(f"Dropped viable regions: {c['dropped_viable']}")
    lines.append("Dropped lb floor: " + ("none" if c["dropped_viable"] == 0 else _g6(outcome["dropped_lb_min"])))
    return lines


def balances(outcome: dict) -> bool:
    """RunTelemetry::balances: every bounded region is pruned or enqueued,
    and every enqueued box (plus the root) was expanded, dropped or is
    pending.  A batched iteration expands many boxes: `expansions` plays
    the reference's per-dequeue `iterations`."""
    c = outcome["counters"]
    bound_flow = c["bounded"] == c["pruned_infeasible"] + c["pruned_dominated"] + c["pruned_duplicate"] + c["enqueued"]
    frontier_flow = (c["enqueued"] + 1 == c["expansions"] + c["dropped_dominated"] + c["dropped_viable"]
                     + outcome["frontier_size"])
    return bool(bound_flow and frontier_flow)
