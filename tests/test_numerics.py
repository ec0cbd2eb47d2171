"""The double-float contraction of the element kernel (csrc/elements.cu: df_split, df_fma,
df_value), restated with numpy float32 arithmetic on the CPU: an FP64 value split into an FP32
pair, exact products by FMA, TwoSum accumulation.  Its error bound (about 2^-46 of the sum of the
absolute terms, against 2^-53 for FP64) is what the element fixtures' 1e-11 tolerance and the
Newton tolerances rely on; the CUDA kernel itself is checked against the reference fixtures in
the GPU parity tests."""

import numpy as np

f32 = np.float32


def _split(d):
    hi = f32(d)
    return hi, f32(np.float64(d) - np.float64(hi))


def _fma(a, b, c):
    # one rounding of a*b + c: exact in float64 for float32 inputs, then rounded to float32
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def _df_fma(acc, a, b):
    (ah, al), (bh, bl) = a, b
    p = f32(ah * bh)
    pe = _fma(ah, bh, -p)
    x = _fma(ah, bl, f32(al * bh))
    s = f32(acc[0] + p)
    bv = f32(s - acc[0])
    err = f32(f32(acc[0] - f32(s - bv)) + f32(p - bv))
    return s, f32(acc[1] + f32(err + f32(pe + x)))


def test_double_float_contraction_error_bound():
    rng = np.random.default_rng(0)
    worst = 0.0
    for t in range(1000):
        n = 8
        u = rng.normal(size=n) * 10 ** rng.uniform(-6, 0)
        g = rng.normal(size=n) * 10 ** rng.uniform(0, 2)
        if t % 2:
            g -= g.mean()  # shape-function gradients sum to zero: cancellation
        acc = (f32(0), f32(0))
        for i in range(n):
            acc = _df_fma(acc, _split(u[i]), _split(g[i]))
        val = np.float64(acc[0]) + np.float64(acc[1])
        worst = max(worst, abs(val - np.dot(u, g)) / np.sum(np.abs(u * g)))
    assert worst < 2.0**-45, worst


def test_split_is_exact_to_48_bits():
    rng = np.random.default_rng(1)
    d = rng.normal(size=10000) * 10.0 ** rng.uniform(-20, 20, size=10000)
    hi = d.astype(np.float32)
    lo = (d - hi.astype(np.float64)).astype(np.float32)
    rel = np.abs(hi.astype(np.float64) + lo.astype(np.float64) - d) / np.abs(d)
    assert rel.max() < 2.0**-47


def test_integer_fp64_fp32_pair_conversions(tmp_path):
    """The integer-only FP64 -> FP32-pair split and FP32 -> FP64 widening of the element kernel's
    double-float operands (edelweissfe_gb300/csrc/dfloat_bits.h), compiled for the host from the
    same source and checked against the compiler's exact conversions on 2 million values and the
    special cases (zero, subnormal, infinity, NaN, out of range)."""
    import os
    import shutil
    import subprocess

    gxx = shutil.which("g++")
    if gxx is None:
        import pytest

        pytest.skip("no C++ compiler")
    here = os.path.dirname(os.path.abspath(__file__))
    exe = str(tmp_path / "dfloat_bits_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", exe, os.path.join(here, "native", "dfloat_bits_check.cpp")],
                   check=True)  # fmt: skip
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "failures 0" in out.stdout


def test_smoothed_aggregation_index_maps(tmp_path):
    """The smoothed-aggregation index maps (edelweissfe_gb300/csrc/amg_sa_pattern.h) and the
    per-thread bodies of the device kernels (edelweissfe_gb300/csrc/amg_sa_body.h, the same source
    compiled for the host): the smoothed prolongator, A P, P^T A P, the restriction and the
    prolongation equal the dense FP64 products to FP32 rounding on random block systems of 3-DOF
    and 6-DOF nodes, with and without masked DOFs, and the dense products vanish outside the
    patterns."""
    import os
    import shutil
    import subprocess

    gxx = shutil.which("g++")
    if gxx is None:
        import pytest

        pytest.skip("no C++ compiler")
    here = os.path.dirname(os.path.abspath(__file__))
    exe = str(tmp_path / "amg_sa_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(here, "native", "amg_sa_check.cpp")], check=True)  # fmt: skip
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "failures 0" in out.stdout
