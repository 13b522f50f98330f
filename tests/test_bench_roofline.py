"""bench.py's roofline arithmetic on the measured phase times (CPU): the
dominant phase against the bound the roofline contract names (HBM for a
transform, with the FP32 pipe beside it as compute_view), and the view of
the same launches' measured DRAM traffic against MEASURED_PEAKS.json."""
import types

import bench


def test_roofline_of_dominant_phase_and_hbm_view():
    cell = types.SimpleNamespace(grid=(120, 120, 120), natoms=216, lmax=2)
    basis = types.SimpleNamespace(ngw=161235, nrods=3577, idxmin=(0, -33, 0), idxmax=(0, 33, 0))
    H = types.SimpleNamespace(precision="mixed_df32", chunk=32)
    prof = {"ft_xyx_vloc": (21.709, 14), "fnl_gemm": (3.632, 1), "enl_hpsi": (4.13, 1),
            "ft_z_bwd": (2.504, 14), "ft_z_fwd": (3.825, 14), "misc": (0.825, 30)}
    peaks = {"hbm_gbs": 6785.5, "bf16_tflops": 1917.4}
    r = bench.roofline_of(H, cell, basis, prof, peaks, 432)
    assert r["kernel"] == "ft_xyx_vloc" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    # algorithmic bytes: Z rows in and out (16 B each) per state, v(r) once
    # per 32-state launch group
    per_state = 2 * 16 * 120 * 3577 + 120 ** 3 * 8 / 32
    launch = per_state * 432 / 14
    assert abs(r["algorithmic_bytes_per_launch"] - launch) < 1e-6 * launch
    assert abs(r["achieved"] - launch / (21.709 / 14 / 1000.0) / 1e9) < 1e-9
    assert abs(r["frac"] - r["achieved"] / 6785.5) < 1e-12
    c = r["compute_view"]
    assert c["pipe"] == "fp32" and abs(c["frac"] - c["achieved"] / 72.2) < 1e-12
    assert 0.4 < c["frac"] < 0.5  # 33.2 of 72.2 measured
    v = r["hbm_view_measured_traffic"]
    assert v["bound"] == "hbm" and v["unit"] == "GB/s" and v["peak"] == 6785.5
    assert abs(v["achieved"] - r["traffic"] / (21.709 / 14 / 1000.0) / 1e9) < 1e-9
    assert abs(r["phase_frac_of_peak"]["fnl_gemm"] - 0.4667) < 2e-3
