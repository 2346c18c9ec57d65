"""The C-ABI library loads without a GPU and exports every symbol of include/gcm.h."""
import ctypes as C

from gpucadforam_gb300 import _native as N


def test_library_exports_every_declared_symbol():
    lib = N.load()
    syms = N.header_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_prototypes_cover_the_header():
    assert set(N.header_symbols()) == set(N.PROTOTYPES)


def test_abi_version_and_status_strings():
    lib = N.load()
    assert lib.gcm_abi_version() == 1
    assert lib.gcm_status_string(0) == b"ok"
    assert lib.gcm_status_string(2) == b"output overflow"


def test_null_arguments_are_rejected_without_a_device():
    lib = N.load()
    assert lib.gcm_ctx_create(0, None) == 1
    assert lib.gcm_ctx_destroy(None) == 0
    assert lib.gcm_mesh_field(None, None, None, 0.0, None, None, 0, None, None) == 1


def test_status_constants_match_the_header():
    import re

    text = open(N.HEADER).read()
    enum = dict((m.group(1), int(m.group(2))) for m in re.finditer(r"\b(GCM_(?:OK|ERR_[A-Z_]+)) = (\d+)", text))
    assert enum and all(getattr(N, k) == v for k, v in enum.items())
    assert {v: k for k, v in enum.items()} == N.STATUS
