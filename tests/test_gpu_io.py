"""Configuration files and HMC checkpoints through the C ABI: the data
section is the reference's host-layout dataset bit for bit, loading checks
group/precision/grid (readConfig's checks) and the checksum, and a chain
resumed from a checkpoint continues exactly as the uninterrupted chain."""
import numpy as np
import pytest

import mesh_gb300 as mg

pytestmark = pytest.mark.gpu

HEADER = 72


@pytest.mark.parametrize("g,p", [(1, 1), (2, 2), (3, 1), (3, 2)])
def test_field_save_load_roundtrip(ctx, tmp_path, g, p):
    dims = [4, 6, 4, 8]
    U = mg.GaugeField(ctx, g, p, mg.Grid(dims)).random(seed=3)
    host = U.export()
    path = str(tmp_path / "cfg.bin")
    U.save(path)
    raw = np.fromfile(path, dtype=mg.real_dtype(p), offset=HEADER)
    np.testing.assert_array_equal(raw, host.ravel())
    info = mg.config_info(path)
    assert info == {"kind": mg.GROUP, "group": g, "precision": p, "dims": dims, "nstack": 4, "trajectory": 0,
                    "seed": 0}
    V = mg.GaugeField(ctx, g, p, mg.Grid(dims)).set_unit().load(path)
    np.testing.assert_array_equal(V.export(), host)
    W = mg.read_config(ctx, path, expected_grid=mg.Grid(dims))
    np.testing.assert_array_equal(W.export(), host)
    assert mg.plaquette(W) == mg.plaquette(U)


def test_load_refuses_mismatch_and_corruption(ctx, tmp_path):
    dims = [4, 4, 4, 8]
    U = mg.GaugeField(ctx, 2, 2, mg.Grid(dims)).random(seed=5)
    path = str(tmp_path / "cfg.bin")
    U.save(path)
    for other, what in ((mg.GaugeField(ctx, 2, 2, mg.Grid([4, 4, 8, 4])), "grid"),
                        (mg.GaugeField(ctx, 3, 2, mg.Grid(dims)), "group"),
                        (mg.GaugeField(ctx, 2, 1, mg.Grid(dims)), "precision"),
                        (mg.Momenta(ctx, 2, 2, mg.Grid(dims)), "group")):
        with pytest.raises(mg.MeshError) as e:
            other.load(path)
        assert e.value.code == 3 and what in str(e.value)
    with pytest.raises(mg.MeshError):
        mg.read_config(ctx, path, expected_grid=mg.Grid([8, 4, 4, 4]))
    b = bytearray(open(path, "rb").read())
    b[HEADER + 100] ^= 0x10
    bad = tmp_path / "bad.bin"
    bad.write_bytes(bytes(b))
    with pytest.raises(mg.MeshError) as e:
        mg.GaugeField(ctx, 2, 2, mg.Grid(dims)).load(str(bad))
    assert "checksum" in str(e.value)
    with pytest.raises(mg.MeshError):
        mg.GaugeField(ctx, 2, 2, mg.Grid(dims)).load(str(tmp_path / "missing.bin"))


@pytest.mark.parametrize("prec", [1, 2])
def test_hmc_checkpoint_resume_is_exact(ctx, tmp_path, prec):
    dims = [4, 4, 6, 8]
    d = mg.make_deltas("2lf", 0.5, 8)
    a = mg.Hmc(ctx, 3, prec, mg.Grid(dims), seed=41)
    a.randomize_gauge_field()
    a.run(5.9, d, 5, use_graph=False)
    b = mg.Hmc(ctx, 3, prec, mg.Grid(dims), seed=41)
    b.randomize_gauge_field()
    b.run(5.9, d, 2, use_graph=True)
    path = str(tmp_path / "chain.bin")
    b.save(path)
    assert mg.config_info(path)["trajectory"] == 2 and mg.config_info(path)["seed"] == 41
    c = mg.Hmc(ctx, 3, prec, mg.Grid(dims), seed=41)
    c.load(path)
    assert c.count == 2
    c.run(5.9, d, 3, use_graph=True)
    np.testing.assert_array_equal(c.U.export(), a.U.export())
    ha, hc = a.history(), c.history()
    np.testing.assert_array_equal(hc["accept_history"][2:], ha["accept_history"][2:])
    np.testing.assert_allclose(hc["plaq_history"][2:], ha["plaq_history"][2:], rtol=1e-13)
    np.testing.assert_array_equal(hc["plaq_history"][:2], 0.0)
    wrong = mg.Hmc(ctx, 3, prec, mg.Grid(dims), seed=42)
    with pytest.raises(mg.MeshError) as e:
        wrong.load(path)
    assert "seed" in str(e.value)
