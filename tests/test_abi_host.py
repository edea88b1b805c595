"""CPU-only checks: the C-ABI library loads and exports every declared symbol; host-side logic
(FD macro table, kernel recognition, `@hide_communication` ranges, argument validation)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from ps_gb300._build import build
    from ps_gb300 import _lib

    build()
    return _lib.load()


def declared_symbols():
    syms = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            syms |= set(re.findall(r"^\s*(?:int|const char\*|void)\s+(ps_\w+)\s*\(", src, flags=re.M))
    return syms


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 19
    for s in sorted(syms):
        assert hasattr(lib, s), s


def test_python_binding_covers_every_symbol():
    from ps_gb300 import _lib

    missing = declared_symbols() - set(_lib.SIGNATURES)
    assert not missing, missing


def test_abi_version_and_no_gpu_behaviour(lib):
    import torch

    assert lib.ps_abi_version() == 1
    n = ctypes.c_int(-1)
    assert lib.ps_device_count(ctypes.byref(n)) == 0
    if torch.cuda.is_available():
        pytest.skip("GPU present: the no-GPU error path is not exercised")
    assert n.value == 0
    rc = lib.ps_init(0)
    assert rc == -6  # PS_ERR_CUDA, with a message, no abort
    from ps_gb300 import _lib

    assert "no CUDA device" in _lib.last_error()
    # entry points fail cleanly before touching the device
    from ps_gb300._lib import PSArray

    a = PSArray(None, (ctypes.c_int64 * 3)(4, 4, 4), 0, 0)
    assert lib.ps_memcopy3d(a, a, a, None, None, 1) == -9  # PS_ERR_NOT_INIT


def test_fd_table_matches_macro_definitions():
    """Spot-check descriptors against src/FiniteDifferences.jl:328-394."""
    from ps_gb300 import fd

    t3 = fd.MACROS[3]
    assert t3["d_xi"] == (fd.DIFF, fd.X, fd.Y | fd.Z)
    assert t3["d2_zi"] == (fd.DIFF2, fd.Z, 7)
    assert t3["av_xyi"] == (fd.AV, fd.X | fd.Y, fd.Z)
    assert t3["harm_yza"] == (fd.HARM, fd.Y | fd.Z, 0)
    assert t3["inn_xz"] == (fd.SEL, 0, fd.X | fd.Z)
    assert fd.MACROS[2]["d2_ya"] == (fd.DIFF2, fd.Y, fd.Y)
    assert fd.MACROS[1]["d2"] == (fd.DIFF2, fd.X, fd.X)
    # every exported macro of the reference modules is present
    assert len(t3) == 9 + 8 + 13 + 13 + 2
    assert len(fd.MACROS[2]) == 8 + 4 + 5 + 5 + 2
    assert len(fd.MACROS[1]) == 8


def test_statement_parsing_and_errors():
    from ps_gb300 import ArgumentError, fd_kernel

    k = fd_kernel("@inn(R) = @d2_yi(A)")
    assert (k.lhs, k.op, k.lhs_inn) == ("inn", "d2_yi", 7)
    with pytest.raises(ArgumentError):
        fd_kernel("@all(R) = @d_xq(A)")
    with pytest.raises(ArgumentError):
        fd_kernel("R = A")
    with pytest.raises(ArgumentError):
        fd_kernel("@inn_xz(R) = @d_xa(A)", ndims=2)


def test_kernel_recognition_from_reference_bodies():
    from ps_gb300 import ArgumentError, kernels

    body = """
        @inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)/dx^2 + @d2_yi(T)/dy^2 + @d2_zi(T)/dz^2));
        return
    """
    assert kernels.from_source(body) is kernels.diffusion3D_step
    flux = """
        @all(qx)   = -lam*@d_xi(T)*_dx                                          # Fourier's law of heat conduction
        @all(qy)   = -lam*@d_yi(T)*_dy                                          # ...
        @all(qz)   = -lam*@d_zi(T)*_dz                                          # ...
        @all(dTdt) = @inn(Ci)*(-@d_xa(qx)*_dx - @d_ya(qy)*_dy - @d_za(qz)*_dz)  # Conservation of energy
        @inn(T2)   = @inn(T) + dt*@all(dTdt)                                    # Update of temperature
        return
    """
    assert kernels.from_source(flux) is kernels.diffusion3D_step_flux
    assert kernels.from_source("@all(T2) = @all(T) + @all(Ci);") is kernels.copy3D
    assert kernels.from_source("@all(R) = @av_xa(A)").op == "av_xa"
    with pytest.raises(ArgumentError):
        kernels.from_source("@all(A) = @all(B)*2; @all(C) = @all(A)")


def test_hide_communication_ranges_match_reference_formula():
    """get_ranges_outer/inner (src/ParallelKernel/hide_communication.jl:350-394) tile the grid."""
    from ps_gb300.kernels import get_ranges_inner, get_ranges_outer

    for ms, bw in [((512, 512, 512), (16, 2, 2)), ((33, 7, 9), (4, 2, 2)), ((20, 14, 12), (1, 1, 1))]:
        cover = np.zeros(ms, dtype=np.int32)
        for lo, hi in get_ranges_outer(bw, ms) + get_ranges_inner(bw, ms):
            cover[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] += 1
        assert np.all(cover == 1)
        outer = get_ranges_outer(bw, ms)
        assert len(outer) == 6
        # the z-boundary slabs come second and third, as the reference's split of comm calls assumes
        assert outer[1][1][2] == bw[2] and outer[2][0][2] == ms[2] - bw[2]
        # different widths at the upper ends (slabs widened to thread blocks) still tile the grid
        uw = (bw[0] + 3, bw[1] + 1, bw[2])
        cover[:] = 0
        for lo, hi in get_ranges_outer(bw, ms, uw) + get_ranges_inner(bw, ms, uw):
            cover[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] += 1
        assert np.all(cover == 1)


def test_ranges_to_box():
    from ps_gb300.kernels import ranges_to_box

    assert ranges_to_box([(1, 10), (2, 5), (1, 1)]) == ([0, 1, 0], [10, 5, 1])
    assert ranges_to_box([range(0, 10), range(3, 4)]) == ([0, 3, 0], [10, 4, 1])


def test_init_argument_validation():
    import ps_gb300 as ps

    with pytest.raises(ps.ArgumentError):
        ps.init_parallel_stencil("CUDA", "Float64", 3)
    with pytest.raises(ps.ArgumentError):
        ps.init_parallel_stencil(ps.GB300, "Float16", 3)
    with pytest.raises(ps.ArgumentError):
        ps.init_parallel_stencil(ps.GB300, "Float64", 4)
    with pytest.raises(ps.NotInitializedError):
        ps.zeros(4, 4, 4) if not ps.is_initialized() else (_ for _ in ()).throw(ps.NotInitializedError())


def test_column_major_check():
    from ps_gb300.core import is_column_major

    assert is_column_major((4, 5, 6), (1, 4, 20))
    assert not is_column_major((4, 5, 6), (30, 6, 1))
    assert is_column_major((1, 5, 6), (99, 1, 5))


def test_hide_communication_widened_slabs():
    """Slabs widened to whole thread blocks: at least the requested widths, the inner box starting
    and ending on block edges, the boxes still tiling the grid; left alone where the grid is too
    small."""
    from ps_gb300.kernels import get_ranges_inner, get_ranges_outer, widened_widths

    for ms, bw in [((512, 512, 512), (16, 2, 2)), ((100, 40, 36), (16, 4, 2)), ((64, 40, 36), (16, 4, 2)),
                   ((300, 131, 7), (3, 1, 1))]:
        lw, hw = widened_widths(bw, ms)
        assert all(lw[d] >= bw[d] and hw[d] >= bw[d] for d in range(3)) and lw[2] == hw[2] == bw[2]
        for d, blk in ((0, 32), (1, 8)):
            if (lw[d], hw[d]) != (bw[d], bw[d]):
                assert lw[d] % blk == 0 and (ms[d] - hw[d]) % blk == 0 and ms[d] > lw[d] + hw[d]
        cover = np.zeros(ms, dtype=np.int8)
        for lo, hi in get_ranges_outer(lw, ms, hw) + get_ranges_inner(lw, ms, hw):
            cover[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] += 1
        assert np.all(cover == 1)
    assert widened_widths((16, 4, 2), (64, 40, 36))[0][0] == 16  # 64 cells: no room to widen x
