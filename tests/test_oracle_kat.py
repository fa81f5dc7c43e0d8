"""The oracle against the reference's own known-answer tests (CPU only).

Pins the CPU restatement before it is trusted as the checker: every analytic
value asserted by the reference's render tests (see tests/kat_cases.py for the
file:line of each) must come out of the oracle.
"""
import pytest

from kat_cases import CASES, run_case


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_known_answers(name, oracle_lib):
    results = run_case(CASES[name], lambda sc, opt: oracle_lib.render(sc, opt, threads=2))
    bad = [label for label, ok in results if not ok]
    assert not bad, f"{name}: failed {bad}"
