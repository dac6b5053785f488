"""GB300-native interval branch-and-bound hot path (CuMINLPSearch)."""

from . import _abi as abi
from .problem import Expr, InvalidDAG, InvalidProblem, Problem, exp, log, pow, sqr, sqrt
from .solver import (Batch, Bounder, CandidateResult, DeviceProblem, Enumerator, OverBudgetError, Sampler, Server,
                     Solver, batch_solve, bisection_choose, compile_program, default_options, eval_boxes,
                     eval_boxes_device, slot_bounds, solve)

__all__ = [
    "abi", "Expr", "Problem", "InvalidDAG", "InvalidProblem", "sqr", "sqrt", "exp", "log", "pow",
    "Bounder", "Sampler", "Enumerator", "CandidateResult", "DeviceProblem", "OverBudgetError", "Solver",
    "default_options", "eval_boxes", "eval_boxes_device", "solve", "Batch", "batch_solve", "Server",
    "bisection_choose", "slot_bounds", "compile_program",
]
