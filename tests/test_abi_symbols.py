"""The C-ABI library builds, loads without a GPU and exports every symbol
that include/pdg.h declares (no compute calls here)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "pdg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pdg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_header_symbols():
    import __graft_entry__
    __graft_entry__.build()
    import pdg
    lib = ctypes.CDLL(pdg.LIB_PATH)
    names = _declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the binding covers every declared symbol
    assert set(names) <= set(pdg._SIGS), set(names) - set(pdg._SIGS)


def test_no_gpu_reports_error_not_crash():
    import torch
    if torch.cuda.is_available():
        return
    import pdg
    try:
        pdg.GridOperator(3, 2, (2, 2, 2))
    except pdg.PDGError as e:
        assert e.status == pdg.PDG_ECUDA
    else:
        raise AssertionError("context creation without a GPU must fail with PDG_ECUDA")


def test_invalid_config_rejected_before_cuda():
    import pdg
    for kw in (dict(dim=4, degree=2, cells=(2, 2, 2)), dict(dim=3, degree=9, cells=(2, 2, 2)),
               dict(dim=3, degree=2, cells=(0, 2, 2))):
        try:
            pdg.GridOperator(**kw)
        except pdg.PDGError as e:
            assert e.status in (pdg.PDG_EINVAL, pdg.PDG_EUNSUPPORTED)
        else:
            raise AssertionError(f"{kw} accepted")
