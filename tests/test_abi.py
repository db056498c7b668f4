"""The C ABI library loads and exports every entry point include/*.h declares; host-side checks that
need no GPU (no compute call is made here)."""
import ctypes
import glob
import os
import re

import jpsolver
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(jp_\w+)\s*\(", text, flags=re.M):
            if not m.group(0).lstrip().startswith("typedef"):
                names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("jp_create", "jp_destroy", "jp_step", "jp_diag", "jp_get_populations", "jp_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(jpsolver.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, "declared in include/*.h but not exported: %s" % missing


def test_binding_covers_every_declared_symbol():
    # every entry point of the header has a ctypes signature in the Python binding
    missing = [n for n in declared_functions() if n not in jpsolver.SIGNATURES]
    assert not missing, missing


def test_abi_version_and_struct_sizes():
    L = jpsolver.lib()
    assert L.jp_abi_version() == 1
    mirrors = [jpsolver.Config, jpsolver.Info, jpsolver.AmrCounts, jpsolver.ServerConfig, jpsolver.Request,
               jpsolver.Result, jpsolver.ServerStats]
    for i, m in enumerate(mirrors):
        assert L.jp_sizeof(i) == ctypes.sizeof(m), m.__name__
    assert L.jp_sizeof(17) == 0


def test_config_defaults_match_reference_flags():
    # uniform: --n 128 --re 1600 --u0 0.05 --tstar 12 (src/tgv3d_uniform.cu:143-147)
    c = jpsolver.config("uniform")
    assert (c.n, c.re, c.u0, c.tstar, c.mb, c.storage) == (128, 1600.0, 0.05, 12.0, 8, 0)
    # amr: --n 32 --re 800 --frac1 .35 --frac2 .35 --l1 all --l2 all --adapt 100 (src/tgv3d_amr.cu:644-674)
    a = jpsolver.config("amr")
    assert (a.n, a.re, a.frac1, a.frac2, a.l1_mode, a.l2_mode, a.adapt_every, a.develop_steps) == \
        (32, 800.0, 0.35, 0.35, 0, 0, 100, 300)
    assert a.max_gb == 0.0


@pytest.mark.parametrize("kw,needle", [
    ({"n": 20}, "N%MB"),                 # the reference exits 2 on N%MB (src/tgv3d_uniform.cu:148)
    ({"n": 0}, "N%MB"),
    ({"mb": 6}, "mb must be"),
    ({"storage": 9}, "storage"),
    ({"re": -1.0}, "re, u0"),
])
def test_invalid_config_rejected_before_device_use(kw, needle):
    with pytest.raises(jpsolver.JPError) as e:
        jpsolver.Solver("uniform", **kw)
    assert e.value.status == 1
    assert needle in str(e.value)


def test_last_error_is_empty_or_string():
    assert isinstance(jpsolver.lib().jp_last_error(), bytes)
