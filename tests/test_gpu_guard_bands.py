"""Guard bands: every array of a kernel call placed in the middle of a larger NaN-filled buffer. A
kernel that reads past one of its arrays then reads NaN, which reaches its outputs (sums, products
and Julia's max/min all propagate it); one that writes past an array overwrites the band. Each
case must give the result of the same call on ordinary arrays, bit for bit, and leave every band
NaN. Sizes: extents that are not multiples of the thread tiles, in both layouts the kernels
choose between (rows of 16-byte multiples, staged by TMA, and not)."""
import numpy as np
import pytest
import torch

import jit_kernels as K

pytestmark = pytest.mark.gpu

GUARD = 4096  # elements on each side of an array (a multiple of 16 bytes for both types)


def _guarded(ps, host):
    """A device array holding `host` (column-major) inside a NaN band of GUARD elements each side;
    returns (array, buffer)."""
    host = np.asfortranarray(host)
    n = host.size
    dt = torch.float64 if host.dtype == np.float64 else torch.float32
    buf = torch.full((2 * GUARD + n,), float("nan"), dtype=dt, device="cuda")
    buf[GUARD:GUARD + n].copy_(torch.from_numpy(host.ravel(order="F")))
    shape = host.shape
    strides = [1]
    for d in shape[:-1]:
        strides.append(strides[-1] * d)
    return buf[GUARD:GUARD + n].as_strided(shape, strides), buf


class _Set:
    """Ordinary and guarded device copies of the same host arrays."""

    def __init__(self, ps, hosts):
        self.plain = [ps.from_host(h) for h in hosts]
        g = [_guarded(ps, h) for h in hosts]
        self.guarded = [a for a, _ in g]
        self.buffers = [b for _, b in g]

    def check(self, ps, which=None):
        for i in (which if which is not None else range(len(self.plain))):
            a, b = ps.to_host(self.plain[i]), ps.to_host(self.guarded[i])
            assert np.array_equal(a, b, equal_nan=True), i
            assert not np.isnan(b).any() or np.isnan(a).any(), i
        for buf in self.buffers:
            assert torch.isnan(buf[:GUARD]).all() and torch.isnan(buf[-GUARD:]).all(), "a write past an array"


def _rand(rng, shape, dt, lo=0.5):
    return (lo + rng.random(shape)).astype(dt)


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("n", [(33, 20, 9), (40, 20, 9)], ids=["odd", "rows16"])
def test_diffusion_forms_and_memcopy(ps, n, dt):
    rng = np.random.default_rng(5)
    for kern in (ps.kernels.diffusion3D_step, ps.kernels.diffusion3D_step_inv, ps.kernels.diffusion3D_step_flux,
                 ps.kernels.diffusion3D_step_flux_lam):
        lam_arr = kern is ps.kernels.diffusion3D_step_flux_lam
        hosts = [np.zeros(n, dt), _rand(rng, n, dt), _rand(rng, n, dt)] + ([_rand(rng, n, dt)] if lam_arr else [])
        for memopt in (False, True):
            s = _Set(ps, hosts)
            for arrs in (s.plain, s.guarded):
                lam = arrs[3] if lam_arr else 0.7
                ps.parallel(kern, arrs[0], arrs[1], arrs[2], lam, 1e-3, 9.0, 11.0, 13.0, memopt=memopt)
            s.check(ps)
    s = _Set(ps, [np.zeros(n, dt), _rand(rng, n, dt), _rand(rng, n, dt)])
    for arrs in (s.plain, s.guarded):
        ps.parallel(ps.kernels.copy3D, *arrs)
    s.check(ps)


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_fd_macro_kernels(ps, dt):
    rng = np.random.default_rng(6)
    n = (36, 20, 11)
    cases = {"@all(R) = @d_xa(A)": (-1, 0, 0), "@inn(R) = @d2_zi(A)": (0, 0, 0), "@all(R) = @av(A)": (-1, -1, -1),
             "@all(R) = @harm_xya(A)": (-1, -1, 0), "@inn(R) = @maxloc(A)": (0, 0, 0),
             "@inn(R) = @av_yzi(A)": (0, 0, 0)}
    for stmt, off in cases.items():
        k = ps.fd_kernel(stmt)
        s = _Set(ps, [np.zeros(tuple(a + b for a, b in zip(n, off)), dt), _rand(rng, n, dt)])
        for arrs in (s.plain, s.guarded):
            ps.parallel(k, *arrs)
        s.check(ps)


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_acoustic3d(ps, dt):
    rng = np.random.default_rng(7)
    n = 21
    shapes = [(n + 1, n, n), (n, n + 1, n), (n, n, n + 1), (n, n, n)]
    hosts = [(rng.random(sh) - 0.5).astype(dt) for sh in shapes]
    s = _Set(ps, hosts + [np.zeros(sh, dt) for sh in shapes])
    for arrs in (s.plain, s.guarded):
        ps.kernels.acoustic3d_step(*arrs, 0.01, 1.0, 1.0, 0.5, 0.5, 0.5)
    s.check(ps)
    s = _Set(ps, hosts)
    for arrs in (s.plain, s.guarded):
        ps.parallel(ps.kernels.acoustic3D_compute_V, *arrs, 0.01, 1.0, 0.5, 0.5, 0.5)
        ps.parallel(ps.kernels.acoustic3D_compute_P, arrs[3], arrs[0], arrs[1], arrs[2], 0.01, 1.0, 0.5, 0.5, 0.5)
    s.check(ps)


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_run_time_compiled_sweeps(ps, dt):
    import bench

    rng = np.random.default_rng(8)
    n = (40, 20, 9)
    k = ps.parallel_kernel(bench.JIT_FLUX_LAM.format(opt=""))
    for memopt in (False, True):
        s = _Set(ps, [np.zeros(n, dt), _rand(rng, n, dt), _rand(rng, n, dt), _rand(rng, n, dt)])
        for arrs in (s.plain, s.guarded):
            ps.parallel(k, *arrs, 1e-3, 9.0, 11.0, 13.0, memopt=memopt)
        s.check(ps)
    k2 = ps.parallel_kernel(K.BLEND3D)
    s = _Set(ps, [np.zeros((n[0] - 2, n[1] - 2, n[2] - 2), dt), _rand(rng, n, dt), _rand(rng, n, dt),
                  _rand(rng, n, dt)])
    for arrs in (s.plain, s.guarded):
        ps.parallel(k2, *arrs, 0.3)
    s.check(ps)


def _swap_fields(obj, fields_cls, names):
    """Replace a Stokes object's arrays by guarded copies; returns the guard buffers."""
    import ps_gb300 as ps
    from ps_gb300.core import descriptor

    bufs = []
    for k in names:
        a, b = _guarded(ps, ps.to_host(obj.arrays[k]))
        obj.arrays[k] = a
        bufs.append(b)
    obj._fields = fields_cls(*[descriptor(obj.arrays[k]) for k in names])
    return bufs


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_stokes_iterations(ps, dt):
    from ps_gb300 import stokes, stokes3d

    nx, ny = 45, 37
    Mus, Rog = stokes.inclusion_setup(nx, ny, 1.0, 1.0, musi=0.1, dtype=dt)
    ref = stokes.Stokes2D(stokes.Stokes2DParams(nx, ny, 1.0, 1.0), Mus, Rog, dtype=dt)
    gd = stokes.Stokes2D(stokes.Stokes2DParams(nx, ny, 1.0, 1.0), Mus, Rog, dtype=dt)
    bufs = _swap_fields(gd, stokes.PSStokes2DFields, stokes.FIELDS)
    for g in (ref, gd):
        g.compute_timesteps()
        g.iterate(7)
    for k in ("Pt", "Vx", "Vy", "txx", "txy", "Rx", "Ry"):
        assert np.array_equal(ref.host(k), gd.host(k)), k
    assert all(torch.isnan(b[:GUARD]).all() and torch.isnan(b[-GUARD:]).all() for b in bufs)

    n = (19, 17, 15)
    Mus3, Rog3 = stokes3d.inclusion_setup(*n, dtype=dt)
    r3 = stokes3d.Stokes3D(stokes3d.Stokes3DParams(*n), Mus3, Rog3, dtype=dt)
    g3 = stokes3d.Stokes3D(stokes3d.Stokes3DParams(*n), Mus3, Rog3, dtype=dt)
    bufs3 = _swap_fields(g3, stokes3d.PSStokes3DFields, stokes3d.FIELDS)
    for g in (r3, g3):
        g.compute_timesteps()
        g.iterate(5)
    for k in ("Pt", "Vx", "Vy", "Vz", "txx", "txy", "tyz", "Rz"):
        assert np.array_equal(r3.host(k), g3.host(k)), k
    assert all(torch.isnan(b[:GUARD]).all() and torch.isnan(b[-GUARD:]).all() for b in bufs3)


def test_adjoint_step(ps):
    rng = np.random.default_rng(9)
    n = (34, 20, 11)
    hosts = [np.zeros(n), rng.standard_normal(n), _rand(rng, n, np.float64), _rand(rng, n, np.float64),
             _rand(rng, n, np.float64), np.zeros(n)]
    s = _Set(ps, hosts)
    for lamT, lamT2, T, Ci, lam, glam in (s.plain, s.guarded):
        ps.adjoint.adjoint_step(lamT, lamT2, T, Ci, lam, glam, 1e-3, 9.0, 11.0, 13.0)
    s.check(ps)
