"""The C-ABI library loads without a GPU and exports every function include/semgb.h declares."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "semgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sem_[a-z0-9_]+)\s*\(", src)))


def test_header_and_library_agree(semgb_lib):
    names = declared()
    assert len(names) >= 30
    lib = semgb_lib.lib()
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(semgb_lib.exported_symbols())


def test_errors_without_gpu_work(semgb_lib):
    import ctypes as C
    lib = semgb_lib.lib()
    h = C.c_void_p()
    assert lib.sem_mesh_create_box(0, 1, 1, 1.0, 1.0, 1.0, 2, C.byref(h)) == semgb_lib.SEM_ERR_ARG
    assert b"box" in lib.sem_last_error_string()
    assert lib.sem_solver_step(None, 1) == semgb_lib.SEM_ERR_ARG
