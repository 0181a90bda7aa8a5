"""CPU-side checks of the C-ABI library: it builds, loads, and exports every
function that include/qaintensor_gb300.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, load_engine

HEADER = os.path.join(ROOT, "include", "qaintensor_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qt_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    eng = load_engine()
    return eng.library()


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("qt_create", "qt_apply_2q", "qt_truncated_svd", "qt_contract_svd", "qt_contract_pair",
                 "qt_switch", "qt_expect_z", "qt_rank_model_train"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_defaults(lib):
    eng = load_engine()
    assert lib.qt_abi_version() == 1
    cfg = eng.QtConfig()
    assert lib.qt_config_default(ctypes.byref(cfg)) == 0
    assert cfg.mode == 0 and cfg.max_sweeps > 0 and cfg.oversample > 0
    assert lib.qt_rank_model_nparams() == 16 * 64 + 64 + 64 * 64 + 64 + 64 + 1


def test_null_arguments_are_rejected_without_a_gpu(lib):
    # argument validation happens before any device work
    assert lib.qt_create(None, None) == -8
    assert lib.qt_mps_site_dims(None, 0, None) == -8
