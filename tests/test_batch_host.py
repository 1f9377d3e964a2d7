"""Host logic of the batching form: the autotuner's search (no GPU)."""
from glint_pipeline_gb300 import GlintError
from glint_pipeline_gb300.batch import autotune


def test_autotune_finds_the_best_setting_and_skips_failures():
    # a cost with its minimum at capacity 128, load factor 0.7, tile width 256;
    # capacity 1024 fails the way a context over its capacities does
    def cost(cfg):
        cap, lf, chunk = cfg
        if cap == 1024:
            raise GlintError(7, "capacity")
        return abs(cap - 128) + 100 * abs(lf - 0.7) + abs(chunk - 256) / 64

    best, table = autotune(lambda c, l, k: (c, l, k), cost)
    assert best[:3] == (128, 0.7, 256)
    assert best[3] == 0
    # capacity x load factor at the first tile width, then the other widths
    assert len(table) == 5 * 3 + 3
    assert all(r["sec_per_step"] == float("inf") for r in table if r["capacity"] == 1024)
    assert {r["refine_chunk"] for r in table[:15]} == {64}
