"""The bench line's roofline arithmetic (algorithmic bytes per launch and per step) on CPU."""

from __future__ import annotations

import bench


def test_config2_passes_move_the_documented_bytes():
    nx, ny, nz = 192, 192, 256
    ncell, nspec = nx * ny * nz, nx * ny * (nz // 2 + 1)
    per_launch = bench.slot_bytes(ncell, nspec, labels=True, nonlinear=True)
    assert len(per_launch) == 8
    # the z velocity pass: three spectra in and out, three velocity fields in and out, the labels
    assert per_launch[3] == 6 * 8 * nspec + 6 * 4 * ncell + ncell == 464_191_488
    assert sum(per_launch) == 1_386_086_400


def test_recording_adds_the_phase_bins_to_the_pressure_pass_only():
    plain = bench.slot_bytes(1000, 600, labels=True, nonlinear=True)
    rec = bench.slot_bytes(1000, 600, labels=True, nonlinear=True, record=True)
    assert [r - p for r, p in zip(rec, plain)] == [0] * 7 + [6 * 4 * 1000]


def test_fused_step_bytes_per_cell():
    assert bench.step_algorithmic_bytes(labels=True, nonlinear=True) == 66
    assert bench.step_algorithmic_bytes(labels=False, nonlinear=False) == 80
    assert bench.step_algorithmic_bytes(labels=False, nonlinear=True) == 84


def test_slot_symbols_name_the_dispatched_kernels():
    assert bench.slot_symbols((192, 192, 256)) == [
        "kf_ypass<192,Y_FWD>", "kf_xpass<192,X_GRAD>", "kf_ypass<192,Y_INV_GRAD>", "kfp_zpass_u<256>",
        "kf_ypass<192,Y_FWD_DIV>", "kf_xpass<192,X_DIV>", "kf_ypass<192,Y_INV>", "kfp_zpass_p<256,false>"]
    # odd ny: per-tile z-passes for lengths with one, runtime-plan passes otherwise
    assert bench.slot_symbols((64, 63, 64))[3] == "kf_zpass_u<64>"
    assert bench.slot_symbols((64, 63, 320))[3] == "k_zpass_u"
    assert bench.slot_symbols((640, 64, 512))[1] == "kf_xpass<640,X_GRAD>"
    # tensor-map staging of the persistent z-tiles (nz / 2 + 1 <= 256 only)
    tma = bench.slot_symbols((192, 192, 256), tma=True)
    assert tma[3] == "kfp_zpass_u<256,true>" and tma[7] == "kfp_zpass_p<256,false,false,true>"
    assert bench.slot_symbols((64, 63, 64), tma=True)[3] == "kf_zpass_u<64>"


def test_pennes_bytes_per_cell_substep():
    # theta, label, q, max, dose, compensation in (4+1+4+4+4+4); theta', max, dose, compensation out (4x4)
    assert bench.PENNES_BYTES_PER_CELL == 21 + 16
