"""The algorithmic byte model of one split-explicit 3D step (the rule: every
distinct 3D operand of a call at pygetm's operator API read once and every
output written once at storage precision, 2D operands per column, interior
cells only).  CPU only."""

import pytest

from getm_gb300 import roofline


def test_fp64_3d_bytes_per_cell_match_the_per_call_rule():
    """FP64: 3D part 2160 B per cell (the reference's call list for the
    seamount: update_depth 256, Momentum.advance 400, update_diagnostics
    816, two tracers 2 x 272, density/pressure/NN 144)."""
    cells = 400 * 300 * 40
    b = roofline.step_bytes(400, 300, 40, "fp64", ntracer=2, split=30)
    assert b["3d"] / cells == pytest.approx(2160.0)
    tr = b["TracerCollection.advance (tracer.py:193-276)"] / cells
    assert tr == pytest.approx(2 * 272.0)  # 4 passes of 48 B, w pass 40 B, diffusion 40 B


def test_mixed_form_stores_less_and_2d_loop_is_form_independent():
    f = roofline.step_bytes(400, 300, 40, "fp64")
    m = roofline.step_bytes(400, 300, 40, "mixed")
    m32 = roofline.step_bytes(400, 300, 40, "mixed", tracer_storage="float32")
    assert m32["3d"] < m["3d"] < f["3d"]
    # FP64 tracer storage: 8 more bytes per tracer read and write in each of
    # the five advection passes and the diffusion, plus the tracers and NN of
    # the density and buoyancy-frequency calls
    cells = 400 * 300 * 40
    assert (m["3d"] - m32["3d"]) / cells == pytest.approx(2 * (5 * 8 + 8) + 2 * 4 + 3 * 4)
    assert m["2d"] == f["2d"]  # every 2D field is float64 in both forms
    assert m["total"] == pytest.approx(m["3d"] + m["2d"])
    # the substep loop: split copies of the per-substep 2D bytes
    sub = roofline.substep_bytes(400, 300)
    assert m["2d"] == pytest.approx(30 * sub + sum(c.per_column for c in roofline.step_calls("mixed")
                                                   if c.count == 1) * 400 * 300)


def test_bytes_scale_with_cells_columns_tracers_and_substeps():
    a = roofline.step_bytes(100, 80, 20, "mixed", ntracer=2, split=30)
    b = roofline.step_bytes(200, 80, 20, "mixed", ntracer=2, split=30)
    assert b["total"] == pytest.approx(2 * a["total"])
    c = roofline.step_bytes(100, 80, 20, "mixed", ntracer=3, split=30)
    d = roofline.step_bytes(100, 80, 20, "mixed", ntracer=2, split=31)
    assert c["3d"] > a["3d"] and c["2d"] == a["2d"]
    assert d["2d"] - a["2d"] == pytest.approx(roofline.substep_bytes(100, 80))
    with pytest.raises(ValueError):
        roofline.step_calls("bf16")
