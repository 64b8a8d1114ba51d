"""The recipe that builds the patched reference (oracle/build_ref.py): a cached
binary is reused only for the configuration it was built for, so every value
the build takes from -D must show in the binary's name."""
import pytest

from oracle import build_ref

BASE = dict(n=(16, 8, 32), k=30, sigma=0.05)


def test_every_build_value_is_in_the_name():
    variants = [
        {}, {"fp64": False}, {"diag": True}, {"setup_b": False}, {"strain": True},
        {"asf": 0.15}, {"cd2": 0.02}, {"d": (1.0, 0.5, 2.0)}, {"d": (2.0, 0.5, 1.0)}, {"dslip": 2.0},
        {"uq2": 0.6}, {"mu": 1.5}, {"lam": 1.0}, {"c11": 6.0}, {"c11": 6.5},
        {"n": (16, 8, 16)}, {"k": 31}, {"sigma": 0.06},
    ]
    names = [build_ref.binary_name(**{**BASE, **v}) for v in variants]
    assert len(set(names)) == len(names), names


def test_default_values_keep_the_short_name():
    plain = build_ref.binary_name(**BASE)
    spelled = build_ref.binary_name(**BASE, d=(1.0, 1.0, 1.0), dslip=1.0, uq2=1.0, mu=1.0, lam=1.5, c11=None)
    assert plain == spelled
    assert "_mu" not in plain and "_C11" not in plain and "_d" not in plain


def test_patches_are_in_line_order_and_name_their_text():
    lines = [ln for ln, _, _ in build_ref.PATCHES]
    assert lines == sorted(lines)
    assert all(old and old != new for _, old, new in build_ref.PATCHES)


def test_patch_set_applies_to_the_reference_source(tmp_path):
    """Every patch finds its original text on its line (the recipe refuses a
    different revision of the reference rather than building something else)."""
    if not build_ref.REF_SRC.exists():
        pytest.skip("no reference checkout here")
    out = build_ref.write_patched_source(dst=tmp_path / "patched.c")
    text = out.read_text(encoding="latin-1")
    for macro in ("PFDD_D1", "PFDD_DSLIP", "PFDD_UQ2", "PFDD_C11", "PFDD_MT"):
        assert f"#define {macro}" in text
