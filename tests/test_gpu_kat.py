"""The reference's known-answer tests through the C-ABI on the GPU."""
import pytest

from kat_cases import CASES, run_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_known_answers(name, gpu_ctx):
    def render(sc, opt):
        b = gpu_ctx.build(sc)
        try:
            return gpu_ctx.render(b, sc, opt)
        finally:
            b.release()
    results = run_case(CASES[name], render)
    bad = [label for label, ok in results if not ok]
    assert not bad, f"{name}: failed {bad}"
