"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/*.h (no GPU calls)."""
import ctypes
import glob
import os
import re

import pytest

from beep_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_entry_points():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        names += re.findall(r"BEEP_API\s+[\w\s\*]+?\b(beep_\w+)\s*\(", src)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared_entry_points()
    assert "beep_simulate" in names and len(names) >= 6
    for n in names:
        assert hasattr(lib, n), n


def test_abi_version():
    build.build()
    assert capi.lib().beep_abi_version() == capi.ABI_VERSION == 4


def test_struct_layout_matches_header():
    # the ctypes mirrors must have the C sizes (checked against a C compile of the header)
    import subprocess, tempfile
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "beep_gpu.h"
int main(void){printf("%zu %zu %zu %zu %zu\n", sizeof(beep_model_desc), sizeof(beep_param_tables),
 sizeof(beep_sim_batch), offsetof(beep_model_desc, obs_cells), offsetof(beep_sim_batch, form));return 0;}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    got = [ctypes.sizeof(capi.ModelDesc), ctypes.sizeof(capi.ParamTables), ctypes.sizeof(capi.SimBatch),
           capi.ModelDesc.obs_cells.offset, capi.SimBatch.form.offset]
    assert [int(x) for x in out] == got


def test_set_option_validates_names_and_values():
    from beep_gb300 import capi
    capi.set_option("fast_foi", capi.FOI_SIMT)
    capi.set_option("fast_foi", capi.FOI_AUTO)
    with pytest.raises(capi.BeepError):
        capi.set_option("fast_foi", 7)
    with pytest.raises(capi.BeepError):
        capi.set_option("no_such_option", 1)
    capi.set_option("sampler_iteration_limit", 1)
    capi.set_option("sampler_iteration_limit", 0)
    for bad in (-1, 65537):
        with pytest.raises(capi.BeepError):
            capi.set_option("sampler_iteration_limit", bad)
