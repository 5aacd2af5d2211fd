"""The C ABI library loads and exports every entry point include/*.h
declares.  No compute call is made (CPU only)."""
import ctypes
import glob
import os
import re

from conftest import REPO


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b(kdgr_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("kdgr_init", "kdgr_scene_create", "kdgr_render", "kdgr_render_trace", "kdgr_render_batch",
                 "kdgr_batch_create", "kdgr_autotune", "kdgr_build_tree", "kdgr_read_kdt", "kdgr_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(pkg.capi.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_error_path_without_gpu_work(pkg):
    L = pkg.capi.lib()
    t = pkg.capi.Tree()
    rc = L.kdgr_read_kdt(b"/nonexistent/file.kdt", ctypes.byref(t))
    assert rc == 4  # KDGR_ERR_IO
    assert b"cannot open" in L.kdgr_last_error()
