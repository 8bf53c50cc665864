"""Configuration rules of the aligner, mirroring the reference's ``cfg::`` namespace.

The reference composes its configuration at compile time as a chain of rules,
each wrapping its predecessor (include/pairwise_aligner/configuration/
rule_base.hpp, rule_category.hpp:24-30), and ``cfg::configure_aligner`` folds the
chain into an aligner object (configure_aligner.hpp:165-206).  The same names
and nesting work here:

    aligner = cfg.configure_aligner(
        cfg.method_global(
            cfg.gap_model_affine(cfg.score_model_unitary_simd_saturated(4, -5), -10, -1),
            cfg.leading_end_gap(), cfg.trailing_end_gap()))
    for r in aligner.compute(seqs1, seqs2):
        r.score()

Every score-model rule of the unitary family (``score_model_unitary``,
``score_model_unitary_simd``, ``score_model_unitary_simd_saturated``) and the
new ``score_model_unitary_gpu`` select the same GB300 kernels: the rule only
carries (match, mismatch); the arithmetic width is chosen per pair on the
device (s16x2 lanes, promoted to s32 when a pair needs it).
"""
from __future__ import annotations

import enum
from dataclasses import dataclass, field
from typing import Any


class end_gap(enum.Enum):
    """cfg::end_gap (end_gap_policy.hpp:20-24)."""
    penalised = False
    free = True


@dataclass(frozen=True)
class leading_end_gap:
    """cfg::leading_end_gap (end_gap_policy.hpp:26-30)."""
    first_column: end_gap = end_gap.penalised
    first_row: end_gap = end_gap.penalised


@dataclass(frozen=True)
class trailing_end_gap:
    """cfg::trailing_end_gap (end_gap_policy.hpp:32-36)."""
    last_column: end_gap = end_gap.penalised
    last_row: end_gap = end_gap.penalised


class rule_category(enum.Enum):
    """cfg::detail::rule_category (rule_category.hpp:24-30)."""
    method = 0
    gap_model = 1
    score_model = 2
    result = 3


@dataclass(frozen=True)
class _Rule:
    category: rule_category | None
    params: dict = field(default_factory=dict)
    predecessor: Any = None

    def chain(self):
        r = self
        while r is not None:
            if r.category is not None:
                yield r
            r = r.predecessor


initial = _Rule(None)


def _split(args, n_params, name):
    """Accept both fn(predecessor, *params) and fn(*params), like the reference CPOs."""
    if len(args) == n_params + 1:
        pred = args[0]
        if not isinstance(pred, _Rule):
            raise TypeError(f"{name}: the predecessor must be a configuration rule")
        return pred, args[1:]
    if len(args) == n_params:
        return initial, args
    raise TypeError(f"{name} takes {n_params} parameters (plus an optional predecessor rule)")


def method_global(*args):
    """cfg::method_global(pred, leading_end_gap, trailing_end_gap) (method_global.hpp:121-145)."""
    if len(args) in (1, 3) and isinstance(args[0], _Rule):
        pred, rest = args[0], args[1:]
    else:
        pred, rest = initial, args
    lead = rest[0] if len(rest) > 0 else leading_end_gap()
    trail = rest[1] if len(rest) > 1 else trailing_end_gap()
    if not isinstance(lead, leading_end_gap) or not isinstance(trail, trailing_end_gap):
        raise TypeError("method_global expects leading_end_gap and trailing_end_gap")
    return _Rule(rule_category.method, {"local": False, "leading": lead, "trailing": trail}, pred)


def method_local(*args):
    """cfg::method_local(pred) (method_local.hpp:118-137); all end gaps are free (:41-49)."""
    pred = args[0] if args else initial
    if len(args) > 1 or not isinstance(pred, _Rule):
        raise TypeError("method_local takes an optional predecessor rule only")
    return _Rule(rule_category.method, {"local": True}, pred)


def gap_model_affine(*args):
    """cfg::gap_model_affine(pred, open, extension) (gap_model_affine.hpp:130-155).

    A gap of length k scores ``open + k * extension`` (both <= 0)."""
    pred, (o, e) = _split(args, 2, "gap_model_affine")
    return _Rule(rule_category.gap_model, {"gap_open": int(o), "gap_extension": int(e)}, pred)


def score_model_unitary_gpu(*args):
    """Unitary substitution scores on the GB300: a == b -> match, else mismatch.

    Same meaning as cfg::score_model_unitary (score_model_unitary.hpp:185-209); raw
    bytes are compared, so case and symbols outside A/C/G/T count as in the reference."""
    pred, (ma, mi) = _split(args, 2, "score_model_unitary_gpu")
    return _Rule(rule_category.score_model, {"match": int(ma), "mismatch": int(mi)}, pred)


# The reference's unitary score models, all routed to the same device kernels.
score_model_unitary = score_model_unitary_gpu
score_model_unitary_simd = score_model_unitary_gpu
score_model_unitary_simd_saturated = score_model_unitary_gpu


def score_model_matrix(*args):
    """cfg::score_model_matrix(pred, matrix) (configuration/score_model_matrix.hpp:203-222).

    ``matrix`` is a sequence of ``(symbol, row)`` pairs, as the reference's
    ``std::array<std::pair<alphabet_t, std::array<score_t, D>>, D>``: the score of a
    sequence1 symbol ``s1`` against a sequence2 symbol ``s2`` is ``row(s1)[rank(s2)]``,
    where the rank of a symbol is its position in the list (score_model/
    score_model_matrix.hpp:53-63).  Up to 32 symbols (single bytes or 1-character
    strings); every symbol of the aligned sequences must be one of them."""
    pred, (matrix,) = _split(args, 1, "score_model_matrix")
    symbols, rows = [], []
    for sym, row in matrix:
        b = sym.encode() if isinstance(sym, str) else (bytes([sym]) if isinstance(sym, int) else bytes(sym))
        if len(b) != 1:
            raise TypeError("score_model_matrix: every symbol must be one byte")
        symbols.append(b[0])
        rows.append([int(x) for x in row])
    dim = len(symbols)
    if not 1 <= dim <= 32 or any(len(r) != dim for r in rows):
        raise ValueError("score_model_matrix: a square matrix of 1..32 symbols is required")
    if len(set(symbols)) != dim:
        raise ValueError("score_model_matrix: symbols must be distinct")
    flat = tuple(x for r in rows for x in r)
    return _Rule(rule_category.score_model, {"match": 0, "mismatch": 0,
                                             "matrix": (bytes(symbols), flat)}, pred)


def band_learned(*args):
    """Opt-in learned band for global alignment: banded DP checked by an admissible
    bound, doubling to the full DP when the bound does not certify the band."""
    pred = args[0] if args else initial
    return _Rule(rule_category.result, {"band_mode": 1}, pred)


def width(*args):
    """Force the arithmetic width (16 or 32) instead of choosing it per pair."""
    pred, (w,) = _split(args, 1, "width")
    return _Rule(rule_category.result, {"width_hint": int(w)}, pred)


def fold(rule: _Rule) -> dict:
    """Collect the chain into one flat configuration (configure_aligner.hpp:136-158)."""
    if not isinstance(rule, _Rule):
        raise TypeError("configure_aligner expects a configuration rule")
    seen: dict = {}
    for r in rule.chain():
        key = (r.category, tuple(sorted(r.params)))
        if r.category in (rule_category.method, rule_category.gap_model, rule_category.score_model):
            if r.category in seen:
                raise TypeError(f"configuration has more than one {r.category.name} rule")
            seen[r.category] = r.params
        else:
            seen.setdefault(key, r.params)
    if rule_category.score_model not in seen:
        raise TypeError("configuration lacks a score model (configure_aligner.hpp:176)")
    if rule_category.gap_model not in seen:
        raise TypeError("configuration lacks a gap model (configure_aligner.hpp:177)")
    method = seen.get(rule_category.method, {"local": False, "leading": leading_end_gap(),
                                             "trailing": trailing_end_gap()})
    out = dict(seen[rule_category.score_model])
    out.update(seen[rule_category.gap_model])
    out["local"] = method["local"]
    if method["local"]:
        out.update(first_column_free=True, first_row_free=True, last_column_free=True, last_row_free=True)
    else:
        lead, trail = method["leading"], method["trailing"]
        out.update(first_column_free=lead.first_column.value, first_row_free=lead.first_row.value,
                   last_column_free=trail.last_column.value, last_row_free=trail.last_row.value)
    out["band_mode"] = 0
    out["width_hint"] = 0
    for k, v in seen.items():
        if isinstance(k, tuple):
            out.update(v)
    return out


def configure_aligner(rule: _Rule, device: int = 0):
    """cfg::configure_aligner (configure_aligner.hpp:165-206) -> an aligner object."""
    from .aligner import Aligner
    return Aligner(fold(rule), device=device)
