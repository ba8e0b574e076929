"""The algorithmic FP64 operation count behind the bench line's roofline
(bench.interior_flops_per_cell_step) equals the operations the oracle
restatement of the reference performs for the same work, counted by
running it under a counting torch function mode (oracle/flop_count.py)."""
import pytest

torch = pytest.importorskip("torch")

import bench  # noqa: E402
from oracle.flop_count import count_step, oracle_kwargs_for  # noqa: E402


def interior_from_counts(counts, D, p, m, update, cells):
    """The k_interior share of the oracle's counted operations: interior
    flux points and their fluxes, the derivative and Picard update, and the
    edge traces each iteration passes to the next; the first iteration's T
    equal time nodes once."""
    nf, T = p + 2, m + 1

    def g(phase):
        return sum(v for (ph, _), v in counts.items() if ph == phase)

    total = 0.0
    for it in range(m + 1):
        share = (1 if it == 0 else T) / T
        total += (g(f"solve_faces[{it}]/apply_axis") * (nf - 2) / nf + g(f"solve_faces[{it}]/compute_primitives")
                  + g(f"solve_faces[{it}]/compute_fluxes")) * share
        if it < m or update == "SD":
            total += (g(f"ader_dudt[{it}]/apply_axis") + g(f"ader_dudt[{it}]/-")) * share
        if it < m:
            total += g(f"solve_faces[{it + 1}]/apply_axis") * 2 / nf
    total += g("ader_predictor[0]/-")
    if update == "SD":
        total += g("ader_update[0]/-")
    return total / cells


@pytest.mark.parametrize("D,p,m,update,N", [(2, 3, 3, "FV", 4), (2, 3, 3, "SD", 4), (3, 2, 2, "FV", 3),
                                             (1, 2, 2, "SD", 8), (2, 2, 1, "FV", 4), (1, 4, 4, "FV", 6)])
def test_interior_count_matches_instrumented_oracle(D, p, m, update, N):
    kw = oracle_kwargs_for(D, p, N, update=update, FB=False)
    kw["m"] = m
    if m != p:
        from spd_gb300.simulator import SDADER_Simulator
        kw["ops"] = SDADER_Simulator.build_operators(p, m)
    counts = count_step(kw)
    want = interior_from_counts(counts, D, p, m, update, N ** D)
    assert bench.interior_flops_per_cell_step(D, p, m, update) == pytest.approx(want, rel=0, abs=1e-9)


def test_headline_count():
    """2D, p = 3, FV update: 40,296 operations per cell and step."""
    assert bench.interior_flops_per_cell_step(2, 3, 3, "FV") == 40296
