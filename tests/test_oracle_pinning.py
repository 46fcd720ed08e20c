"""The oracle restatement pinned against the reference's own code (golden
fixtures generated by tests/golden/make_golden.py from oracle/_ref) and the
reference's own known-answer tests."""
import subprocess

import numpy as np
import pytest

import oracle


def _same(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def test_interp_restatement_is_bit_exact_with_reference(golden):
    for name in golden["interp_names"]:
        n2i = golden[f"interp_{name}_n2i"]
        sp = golden[f"interp_{name}_sparse"]
        d = int(golden[f"interp_{name}_depth"])
        ref = golden[f"interp_{name}_dense"]
        got = oracle.interp_f32(n2i, sp, d)
        assert _same(got, ref), name


def test_interp_fp64_within_1e6_of_reference(golden):
    for name in golden["interp_names"]:
        n2i = golden[f"interp_{name}_n2i"]
        sp = golden[f"interp_{name}_sparse"]
        d = int(golden[f"interp_{name}_depth"])
        ref = golden[f"interp_{name}_dense"].astype(np.float64)
        got = oracle.interp_f64(n2i, sp, d)
        assert np.array_equal(np.isnan(got), np.isnan(ref)), name
        m = ~np.isnan(ref)
        scale = np.abs(sp[(sp != np.float32(1e30))]).max() if (sp != np.float32(1e30)).any() else 1.0
        assert np.all(np.abs(got[m] - ref[m]) <= 1e-6 * np.maximum(np.abs(ref[m]), scale)), name


def test_blend_restatement_matches_reference(golden):
    for i in range(int(golden["blend_count"])):
        dst = golden[f"blend_{i}_dst"].copy()
        ox, oy, just, offx, offy = golden[f"blend_{i}_args"].tolist()
        oracle.blend_image_part(dst, golden[f"blend_{i}_src"], (ox, oy), bool(just), (offx, offy))
        assert np.array_equal(dst, golden[f"blend_{i}_out"]), i


def test_ctf_restatement_matches_reference(golden):
    for i in range(int(golden["ctf_count"])):
        got = oracle.make_ctf(golden[f"ctf_{i}_xs"], golden[f"ctf_{i}_rgba"], int(golden[f"ctf_{i}_count"]))
        assert np.array_equal(got, golden[f"ctf_{i}_out"]), i


@pytest.mark.parametrize("binary", ["ref_kat_b2f", "ref_kat_splitter"])
def test_reference_known_answer_tests_pass(binary):
    exe = oracle.HERE / "_ref" / binary
    if not exe.exists():
        pytest.skip("reference tree not built here (oracle/_ref)")
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
