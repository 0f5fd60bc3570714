"""Slab-depth autotuner: the per-class table, its installation in the
library, the table-building rule, the committed header, and (on a GPU) a
short measurement whose table the solver then uses."""
import os
import re

import numpy as np
import pytest

import fast_gb300 as ft
from fast_gb300 import autotune as at


def _reset():
    for p in at.PRECISIONS:
        for s in at.SOLVERS:
            at.set_slab_table(p, s, None)


@pytest.fixture
def clean_table(monkeypatch):
    monkeypatch.delenv("FAST_TAU_ZC", raising=False)
    _reset()
    yield
    _reset()


def test_size_class_is_log2_of_tile_planes(clean_table):
    # 64 x 8 column tiles: a 64^3 volume has 1 * 8 * 64 = 512 tile-planes (class 9),
    # three right-hand sides of it 1536 (class 10), 1024^3 16 * 128 * 1024 = 2^21.
    assert at.slab_depth((64, 64, 64), 1, ft.Precision.MIXED, ft.DSOLVER_CG)[1] == 9
    assert at.slab_depth((64, 64, 64), 3, ft.Precision.MIXED, ft.DSOLVER_CG)[1] == 10
    assert at.slab_depth((1024, 1024, 1024), 1, ft.Precision.F64, ft.DSOLVER_BICGSTAB)[1] == 21
    # shape (nz, ny, nx) = (7, 9, 65): 2 * 2 * 7 = 28 tile-planes (class 4)
    assert at.slab_depth((7, 9, 65), 1, ft.Precision.F32, ft.DSOLVER_CG)[1] == 4


def test_installed_table_and_override(clean_table, monkeypatch):
    at.set_slab_table(ft.Precision.MIXED, ft.DSOLVER_CG, [6] * 32)
    assert at.slab_depth((128, 128, 128), 1, ft.Precision.MIXED, ft.DSOLVER_CG)[0] == 6
    # other (precision, solver) pairs keep their own table
    other = at.slab_depth((128, 128, 128), 1, ft.Precision.MIXED, ft.DSOLVER_BICGSTAB)[0]
    at.set_slab_table(ft.Precision.MIXED, ft.DSOLVER_CG, None)
    assert at.slab_depth((128, 128, 128), 1, ft.Precision.MIXED, ft.DSOLVER_BICGSTAB)[0] == other
    # a depth is never more than the volume's planes
    at.set_slab_table(ft.Precision.F64, ft.DSOLVER_CG, [64] * 32)
    assert at.slab_depth((10, 40, 40), 1, ft.Precision.F64, ft.DSOLVER_CG)[0] == 10
    monkeypatch.setenv("FAST_TAU_ZC", "16")
    assert at.slab_depth((128, 128, 128), 1, ft.Precision.F64, ft.DSOLVER_CG)[0] == 16


def test_empty_entry_falls_back_to_block_count_rule(clean_table):
    # With no entry, the depth is 32 halved while the launch has < 608 blocks.
    at.set_slab_table(ft.Precision.F32, ft.DSOLVER_CG, [0] * 32)
    for edge, want in ((64, 2), (128, 4), (192, 16), (256, 32)):
        tiles_xy = -(-edge // 64) * -(-edge // 8)
        zc = 32
        while zc > 2 and tiles_xy * -(-edge // zc) < 608:
            zc //= 2
        assert zc == want
        assert at.slab_depth((edge,) * 3, 1, ft.Precision.F32, ft.DSOLVER_CG)[0] == want


def test_bad_arguments_are_rejected(clean_table):
    with pytest.raises(ValueError):
        at.set_slab_table(ft.Precision.F64, ft.DSOLVER_CG, [2000])
    with pytest.raises(ValueError):
        at.set_slab_table(ft.Precision.F64, ft.DSOLVER_CG, [4] * 33)
    with pytest.raises(ValueError):
        at.slab_depth((0, 4, 4), 1, ft.Precision.F64, ft.DSOLVER_CG)


def test_table_from_pools_cases_and_fills_gaps():
    rows = [
        # class 9: depth 4 wins on the pooled time per voxel-iteration
        {"precision": "MIXED", "solver": 1, "class": 9, "voxels": 1000, "s_per_iter": {2: 3e-3, 4: 2e-3, 8: 4e-3}},
        {"precision": "MIXED", "solver": 1, "class": 9, "voxels": 3000, "s_per_iter": {2: 5e-3, 4: 6e-3, 8: 9e-3}},
        # class 12: 8 would win but one case could not run it (stopped early)
        {"precision": "MIXED", "solver": 1, "class": 12, "voxels": 10, "s_per_iter": {8: 1e-3, 16: 2e-3}},
        {"precision": "MIXED", "solver": 1, "class": 12, "voxels": 10, "s_per_iter": {8: None, 16: 3e-3}},
    ]
    t = at.table_from(rows)[("MIXED", 1)]
    assert len(t) == at.NUM_CLASSES
    assert t[9] == 4 and t[12] == 16
    assert t[0] == 4 and t[10] == 4 and t[11] == 16 and t[31] == 16  # nearest measured class
    # a depth measured in only one case of a class does not compete
    rows.append({"precision": "MIXED", "solver": 1, "class": 12, "voxels": 10, "s_per_iter": {16: 2e-3, 64: 1e-4}})
    assert at.table_from(rows)[("MIXED", 1)][12] == 16
    # the block-count rule's depth stays when within the tolerance of the fastest
    near = [{"precision": "F32", "solver": 0, "class": 15, "voxels": 1, "rule_depth": 32,
             "s_per_iter": {16: 1.00, 32: 1.015, 64: 1.05}}]
    assert at.table_from(near)[("F32", 0)][15] == 32
    assert at.table_from(near, tolerance=0.01)[("F32", 0)][15] == 16


def test_render_round_trips_and_committed_header_is_well_formed():
    table = {("F64", 0): list(range(32)), ("MIXED", 1): [8] * 32}
    text = at.render(table, "a GPU", "python -m fast_gb300.autotune --write")
    rows = re.findall(r"\{([0-9, ]+)\},\s*// DSOLVER_", text)
    assert len(rows) == 6
    assert [int(v) for v in rows[0].split(",")] == list(range(32))
    assert [int(v) for v in rows[5].split(",")] == [8] * 32
    with open(at.TABLE_PATH) as f:
        committed = f.read()
    assert "constexpr int kSlabClasses = 32;" in committed
    body = re.findall(r"\{([0-9, ]+)\},\s*// DSOLVER_", committed)
    if body:  # a measured table: six rows of 32 candidate depths
        assert len(body) == 6
        for r in body:
            vals = [int(v) for v in r.split(",")]
            assert len(vals) == 32 and all(v == 0 or v in at.CANDIDATES for v in vals)


@pytest.mark.gpu
def test_measured_table_is_used_by_the_solver(gpu, clean_table, monkeypatch):
    rows = at.measure(cases=[(48, 1)], precisions=[ft.Precision.MIXED], solvers=[ft.DSOLVER_CG],
                      candidates=[2, 8], repeats=1, target_s=0.005)
    assert len(rows) == 1 and set(rows[0]["s_per_iter"]) == {2, 8}
    assert all(v is not None and v > 0 for v in rows[0]["s_per_iter"].values())
    table = at.table_from(rows)
    at.install(table)
    depth = table[("MIXED", 1)][rows[0]["class"]]
    assert at.slab_depth((48, 48, 48), 1, ft.Precision.MIXED, ft.DSOLVER_CG)[0] == depth
    from fast_gb300 import volumes
    m = volumes.spheres((48, 48, 48), seed=5, r_min=3.0, r_max=6.0, solid_fraction=0.5)
    p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-6, precision=ft.Precision.MIXED)
    tuned = ft.get_tortuosity(m, p, ft.DSOLVER_CG)
    monkeypatch.setenv("FAST_TAU_ZC", str(depth))
    forced = ft.get_tortuosity(m, p, ft.DSOLVER_CG)
    assert tuned == forced  # the same depth, the same summation order
    assert tuned > 1.0


def test_cli_merges_timing_files_and_writes_table(tmp_path, clean_table):
    """--from-json a,b: a case in b replaces the same case in a; the written
    header holds the resulting depths."""
    import json

    def row(edge, prec, solver, times):
        return {"edge": edge, "nrhs": 1, "precision": prec, "solver": solver,
                "class": at.slab_depth((edge,) * 3, 1, ft.Precision[prec], ft.DiffusionSolverType(solver))[1],
                "voxels": edge ** 3, "span": 16, "s_per_iter": times}

    a = tmp_path / "a.json"
    b = tmp_path / "b.json"
    a.write_text(json.dumps({"device": "test GPU", "rows": [
        row(128, "MIXED", 1, {"8": 1.0e-3, "16": 2.0e-3}),
        row(64, "F64", 0, {"2": 2.0e-3, "4": 1.0e-3})]}))
    b.write_text(json.dumps({"rows": [row(128, "MIXED", 1, {"8": 3.0e-3, "16": 1.0e-3})]}))
    out = tmp_path / "table.inc"
    assert at.main(["--from-json", f"{a},{b}", "--write", str(out)]) == 0
    text = out.read_text()
    assert "Measured on test GPU" in text
    rows = [[int(v) for v in r.split(",")] for r in re.findall(r"\{([0-9, ]+)\},\s*// DSOLVER_", text)]
    mixed_cg, f64_bicg = rows[5], rows[0]
    assert mixed_cg[12] == 16  # b's timing of the 128^3 case replaced a's
    assert f64_bicg[9] == 4
    assert rows[2] == [0] * 32  # no F32 BiCGSTAB rows: no entries
