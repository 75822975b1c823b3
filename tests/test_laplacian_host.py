"""Host-side contract of the laplacian's C ABI (ctgb_laplacian,
ctgb_laplacian_workspace_size): workspace sizing and the arguments rejected
before any device work. Needs the built library, no GPU."""


def test_laplacian_workspace_contract():
    """ctgb_laplacian_workspace_size: 0 for invalid arguments, grows with n and k,
    256-byte multiples; bounded partial-list buffers."""
    from ctlib_gb300 import _native as N
    lib = N.lib()
    f = lib.ctgb_laplacian_workspace_size
    assert f(0, 4, 1, 0) == 0 and f(10, 0, 1, 0) == 0 and f(10, 4, 0, 0) == 0
    assert f(10, 4, 11, 0) == 0 and f(10, 4, 2, 7) == 0
    a, b = f(1000, 16, 8, 0), f(1000, 16, 16, 0)
    assert 0 < a < b and a % 256 == 0 and b % 256 == 0
    assert f(1000, 16, 8, 1) > a  # fp64 lists are wider
    # dimension does not change the workspace (points are read in place)
    assert f(1000, 3, 8, 0) == f(1000, 300, 8, 0)
    # the partial lists stay bounded (256 MiB) for large n * k
    big = f(1 << 20, 8, 256, 0)
    assert big < (256 << 20) + (1 << 20) * 256 * 8 * 2 + (1 << 24)


def test_laplacian_rejects_bad_arguments_without_gpu_work():
    import ctypes
    from ctlib_gb300 import _native as N
    lib = N.lib()
    ws = ctypes.create_string_buffer(1024)
    # null pointers / bad k are rejected before any device call
    assert lib.ctgb_laplacian(None, 10, 4, 3, 0, None, None, None, 0, None) == N.ERR_INVALID
    assert lib.ctgb_laplacian(ws, 10, 4, 0, 0, ws, ws, ws, 1024, None) == N.ERR_INVALID
    assert lib.ctgb_laplacian(ws, 10, 4, 257, 0, ws, ws, ws, 1024, None) == N.ERR_INVALID
    assert lib.ctgb_laplacian(ws, 10, 4, 3, 5, ws, ws, ws, 1024, None) == N.ERR_INVALID
    assert b"k must be" in lib.ctgb_last_error() or b"laplacian" in lib.ctgb_last_error()
