"""The autotuner (ReadySimulation, grids of >= 2^21 cells) measures, on the
all-zero state, the tile geometry (64x8, 32x16, 128x4) and work-item
height of each half-step kernel and the fused H+E pass against them, and
caches the choice per grid shape, device and build.  Different shapes get
different choices, and whatever it chooses -- and every tile geometry
forced by FDTD_TILE -- gives the oracle's fields bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
CHOICE = ("tile_h", "tile_e", "zchunk_h", "zchunk_e", "fused", "zchunk_f")


def _spec(dims, seed):
    from maxwell_solver_gb300.workloads import GridSpec

    return GridSpec(dims, 40, 8, 3, 4, 30e9, seed)


def _run(spec, steps):
    from maxwell_solver_gb300 import info, simFDTD
    from maxwell_solver_gb300.workloads import setup_grid

    P = setup_grid(simFDTD, spec)
    inf = info(P)
    for f in range(1, 7):  # the trial steps left the state exactly zero
        assert not simFDTD("OutputVis", P, np.uint32(spec.cells), np.int32(f)).any()
    simFDTD("StepN", P, np.int32([0, steps, spec.mode]))
    out = [simFDTD("OutputVis", P, np.uint32(spec.cells), np.int32(f)) for f in range(1, 7)]
    simFDTD("DeleteSimulation", P)
    return inf, out


def _oracle(spec, steps):
    import oracle
    from maxwell_solver_gb300.workloads import grid_materials, grid_source

    I, J, K = spec.dims
    o = oracle.OracleSim("f32")
    o.set_params(pml=spec.pml, tfsf_width=spec.pml + 5)
    o.set_const(np.float32([spec.fctr, spec.delX, spec.delT]), np.int32([spec.steps, I, J, K, 0]))
    eps, sig = grid_materials(spec)
    for f in (1, 2, 3):
        o.update_material(f, sig)
    for f in (4, 5, 6):
        o.update_material(f, eps)
    o.ready_simulation()
    o.init_1d(1.0, grid_source(spec))
    for n in range(steps):
        o.step(n, spec.mode)
    return [o.field(n) for n in FIELDS]


def test_shapes_get_their_own_choices(tmp_path, monkeypatch):
    monkeypatch.setenv("FDTD_TUNE_CACHE", str(tmp_path / "tune.txt"))
    monkeypatch.delenv("FDTD_TILE", raising=False)
    monkeypatch.delenv("FDTD_FUSED", raising=False)
    # narrow, wide, flat, tall and cubic grids of 2.3-5.3 M cells: the
    # measured best tile and item height depend on the shape, so at least
    # two of them differ
    shapes = [(96, 512, 48), (512, 64, 72), (512, 256, 40), (64, 64, 600), (144, 144, 112)]
    choices = []
    for g, dims in enumerate(shapes):
        spec = _spec(dims, 900 + g)
        inf, got = _run(spec, 6)
        choices.append(tuple(inf[k] for k in CHOICE))
        for a, b, n in zip(got, _oracle(spec, 6), FIELDS):
            np.testing.assert_array_equal(a, b, err_msg=f"{dims} {n}")
    assert len(set(choices)) >= 2, choices
    lines = (tmp_path / "tune.txt").read_text().splitlines()
    assert len(lines) == len(shapes) and all(l.startswith("v3 ") for l in lines)


@pytest.mark.parametrize("tile", ["0", "1", "2"])
def test_every_tile_geometry_is_exact(tile, monkeypatch):
    monkeypatch.setenv("FDTD_TILE", tile)
    spec = _spec((70, 44, 52), 950)
    inf, got = _run(spec, 30)
    assert inf["tile_h"] == inf["tile_e"] == int(tile)
    for a, b, n in zip(got, _oracle(spec, 30), FIELDS):
        np.testing.assert_array_equal(a, b, err_msg=n)
