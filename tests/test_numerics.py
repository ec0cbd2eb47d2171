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


def _material_points(rng, n, plastic):
    sig = rng.normal(0.0, 120.0 if plastic else 50.0, (n, 6))
    kap = rng.uniform(0.0, 0.01, n)
    de = rng.normal(0.0, 1e-3, (n, 6)) * rng.uniform(0.0, 2.0, (n, 1))
    de[::7] = 0.0  # the zero-increment shortcut
    de[3::11] *= 1e-16  # below its threshold |de| < 1e-14
    return sig, kap, de


def _run_materials_check(tmp_path, exe, mat, props, sig, kap, de):
    import subprocess

    n = sig.shape[0]
    p8 = np.zeros(8)
    p8[: len(props)] = props
    E, nu = props[0], props[1]
    p8[6] = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))  # lambda and G as the host forms them
    p8[7] = E / (2.0 * (1.0 + nu))
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        f.write(np.array([n, mat], np.int32).tobytes())
        f.write(p8.tobytes())
        f.write(np.hstack([sig, kap[:, None], de]).astype(np.float64).tobytes())
    r = subprocess.run([exe, str(fin), str(fout)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return np.fromfile(fout, np.float64).reshape(n, 17)


def test_element_constitutive_updates_match_oracle(tmp_path):
    """The element kernel's J2 return map and linear elasticity (edelweissfe_gb300/csrc/materials.h),
    compiled for the host from the device source, against the oracle (oracle/materials.py, which
    follows materials/vonmises/vonmises.py:186-254 and linearelastic.py:185-210) point by point:
    stress, kappa and the consistent tangent to 1e-12, for linear and exponential hardening,
    zero increments, and the points where the reference's Newton iteration fails (CutbackRequest)."""
    import os
    import shutil
    import subprocess

    from oracle.materials import ReturnMapFailed, linear_elastic, von_mises

    gxx = shutil.which("g++")
    if gxx is None:
        import pytest

        pytest.skip("no C++ compiler")
    here = os.path.dirname(os.path.abspath(__file__))
    exe = str(tmp_path / "materials_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(here, "native", "materials_check.cpp")], check=True)  # fmt: skip
    Is = np.diag([1.0, 1.0, 1.0, 0.5, 0.5, 0.5])
    one = np.zeros((6, 6))
    one[:3, :3] = 1.0
    rng = np.random.default_rng(7)
    cases = [(1, [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0], True), (1, [210000.0, 0.3, 250.0, 1000.0, 80.0, 30.0], True),
             (1, [210000.0, 0.3, 250.0, 0.0, -240.0, 2e5], True), (0, [210000.0, 0.3], False)]  # fmt: skip
    nFailed = nPlastic = 0
    for mat, props, plastic in cases:
        sig, kap, de = _material_points(rng, 4000, plastic)
        out = _run_materials_check(tmp_path, exe, mat, props, sig, kap, de)
        for p in range(sig.shape[0]):
            try:
                with np.errstate(all="ignore"):
                    if mat == 1:
                        s1, k1, C = von_mises(props, sig[p : p + 1], kap[p : p + 1, None], de[p : p + 1])
                    else:
                        s1, k1, C = linear_elastic(props, sig[p : p + 1], np.zeros((1, 0)), de[p : p + 1])
                        k1 = kap[p : p + 1, None]
            except ReturnMapFailed:
                assert out[p, 0] == 0.0, (props, p)
                nFailed += 1
                continue
            assert out[p, 0] == 1.0, (props, p)
            if not np.all(np.isfinite(s1)):  # the iteration ran into NaN: the kernel flags it
                assert not np.all(np.isfinite(out[p, 1:7]))
                continue
            y = out[p]
            scale = np.max(np.abs(s1)) + 1.0
            assert np.max(np.abs(y[1:7] - s1[0])) <= 1e-12 * scale, (props, p)
            assert abs(y[7] - k1[0, 0]) <= 1e-12 * (abs(k1[0, 0]) + 1e-6), (props, p)
            n = y[11:17]
            Cg = y[8] * one + 2.0 * y[9] * Is - y[10] * np.outer(n, n)
            assert np.max(np.abs(Cg - C[0])) <= 1e-12 * np.max(np.abs(C[0])), (props, p)
            nPlastic += y[10] != 0.0
    assert nFailed > 0 and nPlastic > 1000
