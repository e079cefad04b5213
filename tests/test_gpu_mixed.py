"""Mixed precision (F3D_PREC_MIXED): FP32 splitting, sensor, reconstruction, weights and
viscous fluxes; FP64 state, EOS, metrics/J and RK accumulation.

Tolerances, written per check:
- one RHS against the extended-precision oracle, as error relative to the flux scale (max
  over cells of J * sum |face fluxes| the RHS differences): at most 1.5x the error of the
  reference's own arithmetic (the Float32 restatement with FP64 WENO7 alphas, oracle
  orc32_rhs) on the same inputs, and never required below 2e-6. On noisy or nearly smooth
  stencils FP32 smoothness indicators cancel; the reference's Float32 kernels share that;
- after RK3 steps against the FP64 form through the same library: volume-integrated kinetic
  energy and wall pressure within 1e-5 relative (the mixed-precision target).
"""
import numpy as np
import pytest
import torch

from conftest import rel_linf
from flame3d_mhd_gb300 import cases
from flame3d_mhd_gb300.abi import BC_PERIODIC, PREC_MIXED, make_params
from flame3d_mhd_gb300.solver import Flame3D, side_stream
from oracle import oracle as orc
from test_gpu_parity import curvilinear_coords, dev, host, random_state

pytestmark = pytest.mark.gpu
NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))


def mixed_of(P):
    from flame3d_mhd_gb300.cases import params_copy
    return params_copy(P, precision=PREC_MIXED)


def prepare(P, Q0, x, y, z):
    m, J, Q, U = orc.prepare(P, Q0, x, y, z)
    return m, J, Q, U


CASES = {
    "tgv16_comp": lambda: (lambda c: (c["params"], c["Q"], c["x"], c["y"], c["z"]))(cases.tgv(16, character=0)),
    "tgv16_char": lambda: (lambda c: (c["params"], c["Q"], c["x"], c["y"], c["z"]))(cases.tgv(16, character=1)),
    "sod32_hybrid_char": lambda: (lambda c: (c["params"], c["Q"], c["x"], c["y"], c["z"]))(cases.sod(32, 16, 16)),
    "random_all4_char": lambda: _random(seed=12, spikes=30, phi1=0.02, phi2=0.1, phi3=0.4),
    "random_refbc_viscous": lambda: _random(seed=13, bc="reference", viscous=1, rg=1.0, c_s=1e-2, t_s=1.0),
}


def _random(seed, spikes=0, bc="periodic", **kw):
    if bc == "periodic":
        kw["bc"] = [dict(kind=BC_PERIODIC)] * 6
    P = make_params(24, 16, 12, **kw)
    x, y, z = curvilinear_coords(P)
    return P, random_state(P, seed, spikes), x, y, z


@pytest.mark.parametrize("name", sorted(CASES))
def test_mixed_rhs_vs_fp64_oracle(gpu_lib, name):
    P, Q0, x, y, z = CASES[name]()
    m, J, Q, U = prepare(P, Q0, x, y, z)
    s = Flame3D(mixed_of(P))
    s.set_metrics([dev(a) for a in m], dev(J))
    r = host(s.rhs(dev(Q)))
    s.close()
    rl, scale = orc.rhs_ld(P, Q, m, J)
    r32 = orc.rhs32(P, Q.astype(np.float32), [a.astype(np.float32) for a in m], J.astype(np.float32))
    scaled = max(float(np.abs(r[n][I[1:]] - rl[n][I[1:]]).max() / scale[n]) for n in range(5))
    ref32 = max(float(np.abs(r32[n][I[1:]] - rl[n][I[1:]]).max() / scale[n]) for n in range(5))
    assert scaled <= max(2e-6, 1.5 * ref32), (scaled, ref32, rel_linf(r[I], rl[I]))


def _kinetic_energy(U, J):
    rho = U[0][I[1:]]
    ke = 0.5 * (U[1][I[1:]] ** 2 + U[2][I[1:]] ** 2 + U[3][I[1:]] ** 2) / rho
    return float((ke / J[I[1:]]).sum())


def _run(P, m, J, Q, U, dt, steps):
    s = Flame3D(P)
    s.set_metrics([dev(a) for a in m], dev(J))
    Ud, Und, Qd = dev(U), dev(np.zeros_like(U)), dev(Q)
    with side_stream() as stream:
        s.time_step(Ud, Und, Qd, dt, steps)
    stream.synchronize()
    out = host(Ud), host(Qd)
    s.close()
    return out


def test_mixed_tgv_kinetic_energy_within_1e5(gpu_lib):
    c = cases.tgv(32, character=1)
    P = c["params"]
    m, J, Q, U = prepare(P, c["Q"], c["x"], c["y"], c["z"])
    U64, _ = _run(P, m, J, Q, U, c["dt"], 20)
    U32, _ = _run(mixed_of(P), m, J, Q, U, c["dt"], 20)
    ke64, ke32 = _kinetic_energy(U64, J), _kinetic_energy(U32, J)
    ke0 = _kinetic_energy(U, J)
    assert abs(ke32 - ke64) <= 1e-5 * abs(ke64)
    # and the change of KE over the run (numerical dissipation) is resolved, not noise
    assert abs((ke32 - ke0) - (ke64 - ke0)) <= 1e-2 * abs(ke64 - ke0) + 1e-12 * abs(ke0)
    assert rel_linf(U32[I], U64[I], per_var=False) <= 1e-5


def test_mixed_wall_pressure_within_1e5(gpu_lib):
    """No-slip adiabatic wall at y- (the reference BCs), viscous, hybrid: wall-layer pressure."""
    P, Q0, x, y, z = _random(seed=21, bc="reference", viscous=1, rg=1.0, c_s=1e-3, t_s=1.0)
    m, J, Q, U = prepare(P, Q0, x, y, z)
    dt = 2e-4
    _, Q64 = _run(P, m, J, Q, U, dt, 10)
    _, Q32 = _run(mixed_of(P), m, J, Q, U, dt, 10)
    pw64 = Q64[4, NG:-NG, NG, NG:-NG]  # first interior layer above the y- wall
    pw32 = Q32[4, NG:-NG, NG, NG:-NG]
    assert float(np.abs(pw32 - pw64).max() / np.abs(pw64).max()) <= 1e-5
    assert abs(pw32.mean() - pw64.mean()) <= 1e-5 * abs(pw64.mean())


def test_fp32_rounding_is_the_conversion_instruction(gpu_lib):
    """The mixed form's FP32 copies round FP64 values with integer operations on the IEEE
    layouts: bitwise equal to the conversion instruction (torch's .float()) on random values
    over the whole binary32 range and beyond, exact ties (both parities), the largest finite
    binade, subnormal results, zeros, infinities and NaN."""
    import ctypes as C
    rng = np.random.default_rng(17)
    vals = [rng.standard_normal(2_000_000) * np.exp2(rng.integers(-160, 160, 2_000_000))]
    # exact ties: 29 dropped bits = 1 followed by zeros, even and odd kept mantissas
    m = rng.integers(0, 1 << 23, 200_000, dtype=np.int64)
    e = rng.integers(897, 1151, 200_000, dtype=np.int64)
    ties = ((e << 52) | (m << 29) | (1 << 28)).view(np.float64)
    vals += [ties, -ties, np.nextafter(ties, 0), np.nextafter(ties, np.inf)]
    fmax = float(np.finfo(np.float32).max)
    vals.append(np.array([0.0, -0.0, np.inf, -np.inf, np.nan, fmax, -fmax, fmax * (1 + 2 ** -25),
                          fmax * (1 + 2 ** -24), 2.0 ** -126, 2.0 ** -127, 2.0 ** -149, 2.0 ** -150,
                          1.1754942e-38, 3.4e38, 1e-45, 1e300, -1e-300]))
    x = np.concatenate(vals)
    xd = torch.from_numpy(x).cuda()
    out = torch.empty(x.size, dtype=torch.float32, device="cuda")
    rc = gpu_lib.f3d_debug_round_f32(C.c_void_p(xd.data_ptr()), C.c_void_p(out.data_ptr()), x.size, None)
    assert rc == 0
    ref = xd.float()
    torch.cuda.synchronize()
    a, b = out.cpu().numpy().view(np.uint32), ref.cpu().numpy().view(np.uint32)
    nan = np.isnan(ref.cpu().numpy())
    assert np.array_equal(a[~nan], b[~nan])
    assert np.isnan(out.cpu().numpy()[nan]).all()
