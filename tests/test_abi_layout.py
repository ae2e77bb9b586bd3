"""The ctypes mirrors of include/mrg.h's parameter structs (mri_recon_gb300/_lib.py) have the
header's sizes and field offsets: a C program compiled against the header prints them.  A
field added to one side only would make the library read or write past the caller's struct."""
import ctypes
import os
import subprocess

from tests.conftest import ROOT

STRUCTS = {"mrg_config": "MrgConfig", "mrg_dcf_params": "MrgDcfParams", "mrg_fista_params": "MrgFistaParams",
           "mrg_clear_params": "MrgClearParams", "mrg_espirit_params": "MrgEspiritParams"}


def test_struct_layouts_match_header(tmp_path):
    import mri_recon_gb300._lib as L
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "mrg.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in getattr(L, pyname)._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.splitlines())
    for cname, pyname in STRUCTS.items():
        cls = getattr(L, pyname)
        assert int(got[cname + " size"]) == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got[cname + "." + fname]) == getattr(cls, fname).offset, cname + "." + fname
