"""CPU tests of the drop-in programs' host logic: CLI, file names, box I/O, parameters."""
import os

import numpy as np
import pytest

from conftest import module

boxio = module("tocmfastpy.boxio")
fhb = module("Programs.find_HII_bubbles")
dtp = module("Programs.delta_T")
common = module("Programs._common")


def test_output_name_follows_reference_format():
    p = common.params({"ZETA": 30.0, "ION_Tvir_MIN": 1e4, "R_BUBBLE_MAX": 15.0})
    name = fhb.output_name(8.0, 0.343186, p, 0, 64, 100)
    # find_HII_bubbles.py:227-228
    assert name == "xH_nohalos_z8.00_nf0.343186_eff30.0_HIIfilter0_Tvirmin10000.0_RHIImax15_64_100Mpc.npy"
    back = boxio.parse_filename(name)
    assert back["z"] == 8.0 and back["nf"] == pytest.approx(0.343186) and back["eff"] == 30.0
    assert back["HIIdim"] == 64 and back["BoxSize"] == 100 and back["type"] == "xh"


def test_cli_options_and_types():
    o = fhb.parser().parse_args(["-f", "0", "-u", "1", "-z", "9.5", "-q", "box.npy"])
    assert (o.FILTER_TYPE, o.UPDATE_TYPE, o.Z, o.QUIET, o.args) == (0, 1, 9.5, True, ["box.npy"])
    d = fhb.parser().parse_args([])
    assert d.FILTER_TYPE == 1 and d.UPDATE_TYPE == 0 and d.Z == 12.0     # INIT_PARAMS defaults


def test_unknown_parameter_names_are_rejected():
    with pytest.raises(KeyError):
        common.params({"ZETAA": 3})
    c = common.cosmo_of(common.params())
    assert c.omega_M_0 == 0.315 and c.h == 0.673


def test_raw_boxes_plain_and_fftw_padded(tmp_path):
    n = 8
    box = np.arange(n ** 3, dtype=np.float32).reshape(n, n, n)
    plain = tmp_path / "updated_smoothed_deltax_z8.00_8_20Mpc"
    box.tofile(plain)
    b = boxio.readbox(str(plain))
    assert np.array_equal(b.box_data, box) and b.param_dict["type"] == "density"
    padded = np.zeros((n, n, 2 * (n // 2 + 1)), np.float32)
    padded[:, :, :n] = box
    pf = tmp_path / "xH_nohalos_z8.00_nf0.5_eff30.0_8_20Mpc"
    padded.tofile(pf)
    assert np.array_equal(boxio.readbox(str(pf)).box_data, box)
    bad = tmp_path / "deltax_z0.00_8_20Mpc"
    np.zeros(100, np.float32).tofile(bad)
    with pytest.raises(boxio.BoxFormatError):
        boxio.readbox(str(bad))
    with pytest.raises(FileNotFoundError):
        boxio.find_files(str(tmp_path), "nothing*")
    assert len(boxio.find_files(str(tmp_path), "*Mpc")) == 3


def test_delta_T_finds_density_under_every_reference_name(tmp_path):
    os.makedirs(tmp_path / "Boxes")
    d = np.ones((8, 8, 8), np.float32)
    for name in ["updated_smoothed_deltax_z08.00_8_20Mpc.npy", "updated_smoothed_deltax_z8.00_8_20Mpc.npy",
                 "updated_smoothed_deltax_z008.00_8_20Mpc.npy"]:
        np.save(tmp_path / "Boxes" / name, d)
        got = dtp._density_for(str(tmp_path), 8.0, 8, 20.0)
        assert got.shape == (8, 8, 8)
        os.remove(tmp_path / "Boxes" / name)
    with pytest.raises(FileNotFoundError):
        dtp._density_for(str(tmp_path), 8.0, 8, 20.0)


def test_engine_calls_need_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(Exception):
        fhb.conv_bubbles(np.zeros((32, 32, 32), np.float32), {"BoxSize": 48, "HIIdim": 32, "z": 8.0},
                         fil=0, quiet=True, params={"ZETA": 30.0})


def test_run_boxes_and_box_fields(tmp_path, capsys):
    names = ["xH_nohalos_z8.00_nf0.5_eff30.0_8_20Mpc", "xH_nohalos_z9.00_nf0.7_eff30.0_8_20Mpc",
             "xH_nohalos_z9.00_nf0.7_eff30.0_16_20Mpc", "delta_T_z8.00_8_20Mpc"]
    for n in names:
        np.zeros((8, 8, 8), np.float32).tofile(tmp_path / n)
    run = boxio.find_run_boxes(str(tmp_path / names[1]))
    assert [os.path.basename(f) for f in run] == sorted(names[:2])
    b = boxio.readbox(str(tmp_path / names[0]))
    assert "'nf': 0.5" in capsys.readouterr().out          # the reference prints the parameters
    assert b.dim == 8 and b.z == 8.0 and b.init and b.box_data.shape == (8, 8, 8)
    boxio.readbox(str(tmp_path / names[0]), quiet=True)
    assert capsys.readouterr().out == ""
    c = boxio.Box()
    c.setBox(b.box_data, b.param_dict)
    assert c.init and c.dim == 8
    with pytest.raises(boxio.BoxFormatError):
        boxio.find_run_boxes(str(tmp_path / "no_size_field"))
