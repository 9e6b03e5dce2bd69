"""Host logic of the 2D tuning tool (no GPU): the ptxas report parser, the
choice rule and the table writer, which must produce a header that compiles
to the same table."""
import os
import shutil

from perks_gb300 import autotune as A

PTXAS = """ptxas info    : Compiling entry function '_ZN5perks16stencil2d_kernelIfLi1ELb0ENS_6Cfg2DTIfLi1ELi12ELi6ELi0EEEEEvNS_15Stencil2DParamsE' for 'sm_103a'
ptxas info    : Function properties for _ZN5perks16stencil2d_kernelIfLi1ELb0ENS_6Cfg2DTIfLi1ELi12ELi6ELi0EEEEEvNS_15Stencil2DParamsE
    0 bytes stack frame, 0 bytes spill stores, 0 bytes spill loads
ptxas info    : Used 168 registers, used 1 barriers
ptxas info    : Function properties for _ZN5perks16stencil2d_kernelIfLi6ELb0ENS_6Cfg2DTIfLi6ELi8ELi6ELi0EEEEEvNS_15Stencil2DParamsE
    16 bytes stack frame, 12 bytes spill stores, 12 bytes spill loads
ptxas info    : Used 128 registers, used 1 barriers
"""


def test_ptxas_report():
    r = A.ptxas_report(PTXAS)
    assert r == {1: {"spill": 0, "regs": 168}, 6: {"spill": 12, "regs": 128}}


def test_choose_needs_a_wider_margin_to_spill_more():
    spills = {"s2d_f32_ref_default": {1: {"spill": 0}, 6: {"spill": 12}},
              "s2d_f32_ref_nw16_d4_fin1_rp1": {1: {"spill": 0}, 6: {"spill": 40}},
              "s2d_f32_ref_nw8_d6_fin0_rp1": {1: {"spill": 0}, 6: {"spill": 0}}}
    res = {"f32/ref/2ds9pt": {"default": {"gcells": 700.0}, "s2d_f32_ref_nw16_d4_fin1_rp1": {"gcells": 750.0},
                              "s2d_f32_ref_nw8_d6_fin0_rp1": {"gcells": 705.0}},
           "f32/ref/2d9pt": {"default": {"gcells": 100.0}, "s2d_f32_ref_nw16_d4_fin1_rp1": {"gcells": 104.0},
                             "s2d_f32_ref_nw8_d6_fin0_rp1": {"error": "output differs from the built-in kernel"}},
           "f32/ref/2d5pt": {"default": {"gcells": 100.0}, "s2d_f32_ref_nw16_d4_fin1_rp1": {"gcells": 100.5}}}
    t = A.choose(res, spills, margin=0.01)
    assert t["f32/ref/2ds9pt"]["nw"] == 16 and t["f32/ref/2ds9pt"]["fin"] == 1
    assert "f32/ref/2d9pt" not in t  # +4 % with more spills is not enough; the other is wrong
    assert "f32/ref/2d5pt" not in t  # within the noise margin
    # JSON round trips turn the shape keys into strings
    sj = {n: {str(k): v for k, v in d.items()} for n, d in spills.items()}
    assert A.choose(res, sj, margin=0.01) == t


def test_write_table_roundtrip(tmp_path):
    dst = tmp_path / "tune2d.cuh"
    shutil.copy(A.TABLE, dst)
    t = {"f32/ref/2ds9pt": {"nw": 16, "d": 4, "fin": 1, "rp": 2, "nv": 1},
         "f64/fast/2d25pt": {"nw": 8, "d": 3, "fin": 0, "rp": 0, "nv": 0}}
    A.write_table(t, str(dst))
    text = dst.read_text()
    body = text[text.index("// BEGIN TABLE"):text.index("// END TABLE")]
    rows = [r for r in body.split("\n") if "{" in r]
    # f32 ref row, second shape; f64 fast row, last shape
    assert "{0, 0, 0, 0, 0}, {16, 4, 1, 2, 1}, {0, 0, 0, 0, 0}" in rows[1]
    assert rows[-1].rstrip().endswith("{8, 3, 0, 0, 0}}}};")
    assert text.count("{") - text.count("}") == 0
    assert A.read_table(str(dst)) == t


def test_merge_keeps_entries_without_a_winner(tmp_path):
    dst = tmp_path / "tune2d.cuh"
    shutil.copy(A.TABLE, dst)
    A.write_table({"f32/ref/2d5pt": {"nw": 16, "d": 4, "fin": 1, "rp": 0, "nv": 0},
                   "f64/ref/2d21pt": {"nw": 12, "d": 6, "fin": 0, "rp": 0, "nv": 0}}, str(dst))
    assert A.read_table(str(dst))["f64/ref/2d21pt"]["nw"] == 12
    # a new measurement against the table's kernels: only 2ds9pt has a winner
    m = A.merge_table(str(dst), "2d", {"f32/ref/2ds9pt": {"nw": 12, "d": 6, "fin": 0, "rp": 2, "nv": 1, "gcells": 1.0}})
    assert m["f32/ref/2d5pt"] == {"nw": 16, "d": 4, "fin": 1, "rp": 0, "nv": 0}
    assert m["f32/ref/2ds9pt"] == {"nw": 12, "d": 6, "fin": 0, "rp": 2, "nv": 1}
    assert m["f64/ref/2d21pt"] == {"nw": 12, "d": 6, "fin": 0, "rp": 0, "nv": 0}


def test_merge_keeps_the_table_value_of_a_knob_swept_as_zero(tmp_path):
    dst = tmp_path / "tune2d.cuh"
    shutil.copy(A.TABLE, dst)
    A.write_table({"f32/ref/2d5pt": {"nw": 16, "d": 4, "fin": 1, "rp": 2, "nv": 1}}, str(dst))
    # only the division form was swept; the other knobs ran at their table values
    m = A.merge_table(str(dst), "2d", {"f32/ref/2d5pt": {"nw": 0, "d": 0, "fin": 0, "rp": 0, "nv": 0, "gcells": 1.0}})
    assert m["f32/ref/2d5pt"] == {"nw": 16, "d": 4, "fin": 0, "rp": 2, "nv": 1}


def test_3d_table_roundtrip(tmp_path):
    dst = tmp_path / "tune3d.cuh"
    shutil.copy(A.KINDS["3d"]["table"], dst)
    A.write_table({"f64/fast/poisson": {"nwc": 8, "ry": 2, "dkb": 96}}, str(dst), "3d")
    assert A.read_table(str(dst), "3d") == {"f64/fast/poisson": {"nwc": 8, "ry": 2, "dkb": 96}}
    assert A.parse_variant("s3d_f64_fast_nwc8_ry2_dkb96") == {"nwc": 8, "ry": 2, "dkb": 96}


def test_committed_tables_are_in_range():
    """Every entry of the committed tables names a setting the kernels build:
    a value outside these ranges (say a division form of 4) would compile to
    some other form without an error."""
    for key, e in A.read_table(A.TABLE, "2d").items():
        assert e["nw"] == 0 or 1 <= e["nw"] <= 32, (key, e)
        assert e["d"] == 0 or 1 <= e["d"] <= 8, (key, e)
        assert 0 <= e["fin"] <= 3, (key, e)
        assert e["rp"] in (0, 1, 2), (key, e)
        assert 0 <= e["nv"] <= 3, (key, e)
        if "/fast/" in key:
            assert e["fin"] == 0, key  # fast order has no division
    for key, e in A.read_table(A.KINDS["3d"]["table"], "3d").items():
        assert e["nwc"] == 0 or 1 <= e["nwc"] <= 31, (key, e)
        assert e["ry"] >= 0 and e["dkb"] >= 0, (key, e)
