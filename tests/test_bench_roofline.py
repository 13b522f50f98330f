"""bench.py's roofline arithmetic on the measured phase times (CPU): the
dominant phase, its fraction of the pipe peak, and the HBM view of the same
launches against MEASURED_PEAKS.json's copy bandwidth."""
import types

import bench


def test_roofline_of_dominant_phase_and_hbm_view():
    cell = types.SimpleNamespace(grid=(120, 120, 120), natoms=216, lmax=2)
    basis = types.SimpleNamespace(ngw=161235, nrods=3577, idxmin=(0, -33, 0), idxmax=(0, 33, 0))
    H = types.SimpleNamespace(precision="mixed_df32")
    prof = {"ft_xyx_vloc": (21.709, 14), "fnl_gemm": (3.632, 1), "enl_hpsi": (4.13, 1),
            "ft_z_bwd": (2.504, 14), "ft_z_fwd": (3.825, 14), "misc": (0.825, 30)}
    peaks = {"hbm_gbs": 6785.5, "bf16_tflops": 1917.4}
    r = bench.roofline_of(H, cell, basis, prof, peaks, 432)
    assert r["kernel"] == "ft_xyx_vloc" and r["bound"] == "fp32"
    assert abs(r["frac"] - r["achieved"] / 72.2) < 1e-12
    assert 0.4 < r["frac"] < 0.5  # 33.2 of 72.2 measured
    v = r["hbm_view"]
    assert v["bound"] == "hbm" and v["unit"] == "GB/s" and v["peak"] == 6785.5
    assert abs(v["achieved"] - r["traffic"] / (21.709 / 14 / 1000.0) / 1e9) < 1e-9
    assert abs(r["phase_frac_of_peak"]["fnl_gemm"] - 0.4667) < 2e-3
