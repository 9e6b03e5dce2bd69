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


def test_choose_keeps_builtin_unless_faster_and_no_more_spills():
    spills = {"s2d_f32_ref_default": {1: {"spill": 0}, 6: {"spill": 12}},
              "s2d_f32_ref_nw16_d4_f1": {1: {"spill": 0}, 6: {"spill": 40}},
              "s2d_f32_ref_nw8_d6_f0": {1: {"spill": 0}, 6: {"spill": 0}}}
    res = {"f32/ref/2ds9pt": {"default": {"gcells": 700.0}, "s2d_f32_ref_nw16_d4_f1": {"gcells": 750.0},
                              "s2d_f32_ref_nw8_d6_f0": {"gcells": 705.0}},
           "f32/ref/2d9pt": {"default": {"gcells": 100.0}, "s2d_f32_ref_nw16_d4_f1": {"gcells": 200.0},
                             "s2d_f32_ref_nw8_d6_f0": {"error": "output differs from the built-in kernel"}}}
    t = A.choose(res, spills, margin=0.01)
    assert t["f32/ref/2ds9pt"]["nw"] == 16 and t["f32/ref/2ds9pt"]["fin"] == 1
    assert "f32/ref/2d9pt" not in t  # the faster one spills more; the other is wrong


def test_write_table_roundtrip(tmp_path):
    dst = tmp_path / "tune2d.cuh"
    shutil.copy(A.TABLE, dst)
    A.write_table({"f32/ref/2ds9pt": {"nw": 16, "d": 4, "fin": 1}, "f64/fast/2d25pt": {"nw": 8, "d": 3, "fin": 0}},
                  str(dst))
    text = dst.read_text()
    body = text[text.index("// BEGIN TABLE"):text.index("// END TABLE")]
    rows = [r for r in body.split("\n") if "{" in r]
    # f32 ref row, second shape; f64 fast row, last shape
    assert "{0, 0, 0}, {16, 4, 1}, {0, 0, 0}" in rows[1]
    assert rows[-1].rstrip().endswith("{8, 3, 0}}}};")
    assert text.count("{") - text.count("}") == 0
