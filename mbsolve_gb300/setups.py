"""Scenario builders: the reference command-line tool's presets
(mbsolve-tool/src/mbsolve-tool.cpp:163-664) and the benchmark workloads.

Each builder returns (device, scenario) using the mbsolve-style API of
mbsolve_gb300.lib. Material ids get a per-call suffix so that repeated
calls do not collide in the global material library.
"""
import itertools
import math

import numpy as np

from . import lib as mb

_uid = itertools.count()


def _material(base, qm=None, *args):
    m = mb.material("%s#%d" % (base, next(_uid)), qm, *args)
    mb.material.add_to_library(m)
    return m


def _courant_endtime(n_x, length, n_t, eps_r=1.0):
    """End time that gives exactly n_t steps at Courant number 0.5 on an
    n_x-point grid over `length` (common_fdtd.hpp:95-110)."""
    dx = length / (n_x - 1)
    v = 1.0 / math.sqrt(mb.MU0 * mb.EPS0 * eps_r)
    dt = 0.5 * dx / v
    return (n_t - 1.5) * dt


# --------------------------------------------------- reference presets

def ziolkowski1995(num_gridpoints=32768, endtime=200e-15):
    """Self-induced transparency, 2-level (mbsolve-tool.cpp:249-308)."""
    qm = mb.qm_desc_2lvl(1e24, 2 * mb.PI * 2e14, 6.24e-11, 1.0e10, 1.0e10)
    vac = _material("Vacuum")
    ar = _material("AR_Ziolkowski", qm)
    dev = mb.device("Ziolkowski")
    dev.add_region(mb.region("Vacuum left", vac, 0, 7.5e-6))
    dev.add_region(mb.region("Active region", ar, 7.5e-6, 142.5e-6))
    dev.add_region(mb.region("Vacuum right", vac, 142.5e-6, 150e-6))
    sce = mb.scenario("Basic", num_gridpoints, endtime,
                      mb.ic_density_const(mb.qm_operator([1, 0, 0])),
                      mb.ic_field_const(0.0))
    sce.add_source(mb.sech_pulse("sech", 0.0, mb.source.hard_source,
                                 4.2186e9, 2e14, 10, 2e14))
    sce.add_record(mb.record("inv12", 2.5e-15))
    sce.add_record(mb.record("e", 2.5e-15))
    return dev, sce


def song2005(endtime=80e-15, num_timesteps=10000):
    """0-D V-type 3-level system (mbsolve-tool.cpp:163-248)."""
    H = mb.qm_operator([0, 2.3717 * mb.HBAR * 1e15, 2.4165 * mb.HBAR * 1e15])
    u = mb.qm_operator([0, 0, 0], [-mb.E0 * 9.2374e-11,
                                   -mb.E0 * 9.2374e-11 * math.sqrt(2), 0])
    rate = 1e10
    relax = mb.qm_lindblad_relaxation(
        [[0, rate, rate], [rate, 0, rate], [rate, rate, 0]], [0, 0, 0])
    qm = mb.qm_description(6e24, H, u, relax)
    ar = _material("AR_Song", qm)
    dev = mb.device("Song")
    dev.add_region(mb.region("Active region (single point)", ar, 0, 0))
    sce = mb.scenario("Basic", 1, endtime,
                      mb.ic_density_const(mb.qm_operator([1, 0, 0])),
                      mb.ic_field_const(0.0), mb.ic_field_const(0.0),
                      num_timesteps)
    sce.add_source(mb.sech_pulse("sech", 0.0, mb.source.hard_source, 3.5471e9,
                                 3.8118e14, 17.248, 1.76 / 5e-15, -mb.PI / 2))
    for i in (1, 2, 3):
        sce.add_record(mb.record("d%d%d" % (i, i), mb.record.density, i, i,
                                 0, 0))
    sce.add_record(mb.record("e", 0, 0.0))
    return dev, sce


def marskar2011(N=6, num_gridpoints=8192, endtime=2e-12, length=1e-3):
    """N-level anharmonic ladder, Gaussian pulse (mbsolve-tool.cpp:
    479-662). The records sit at x = 0, where the hard source fixes the
    field, so a shorter device with the same grid spacing (length =
    1e-3 (num_gridpoints - 1) / 8191) gives the same records."""
    energies = [0.0] * N
    for i in range(1, N):
        energies[i] = energies[i - 1] + \
            (1.0 - 0.1 * (i - 3)) * mb.HBAR * 2 * mb.PI * 1e13
    H = mb.qm_operator(energies)
    dipoles = []
    for i in range(1, N):
        dipoles += [0.0] * (i - 1) + [-1e-29]
    u = mb.qm_operator([0.0] * N, dipoles)
    T = 600
    pure_deph = 1e12
    scat, deph = [], []
    for i in range(N):
        row = []
        for j in range(N):
            if i == j:
                rate = 0.0  # overwritten by the relaxation constructor
            elif i == j - 1:
                rate = 1e12 / (1 + 0.1 * i)
            elif i == j + 1:
                rate = 1e12 / (1 + 0.1 * j) * \
                    math.exp((energies[j] - energies[i]) / (mb.KB * T))
            else:
                rate = 0.0
            row.append(rate)
            deph.append(pure_deph)
        scat.append(row)
    relax = mb.qm_lindblad_relaxation(scat, deph)
    qm = mb.qm_description(1e25, H, u, relax)
    ar = _material("AR_Marsk", qm)
    dev = mb.device("marskar2011-%dlvl" % N)
    dev.add_region(mb.region("Active region", ar, 0, length))
    total = 0.0
    for i in range(N):
        prod = 1.0
        for j in range(i):
            prod *= scat[j + 1][j] / scat[j][j + 1]
        total += prod
    pops = [1 / total]
    for i in range(1, N):
        pops.append(pops[i - 1] * scat[i][i - 1] / scat[i - 1][i])
    sce = mb.scenario("basic", num_gridpoints, endtime,
                      mb.ic_density_const(mb.qm_operator(pops)),
                      mb.ic_field_const(0.0))
    tau = 100e-15
    sce.add_source(mb.gaussian_pulse("gaussian", 0.0, mb.source.hard_source,
                                     5e8, 1e13, 3.0 * tau, tau))
    for i in range(1, N + 1):
        sce.add_record(mb.record("d%d%d" % (i, i), mb.record.density, i, i,
                                 0.0, 0.0))
    sce.add_record(mb.record("e", mb.record.electric, 0, 0, 0.0, 0.0))
    return dev, sce


def tzenov2016(num_gridpoints=8192, endtime=0.2e-9, mirror=False,
               seed=None, length=5e-3):
    """Quantum cascade laser frequency comb, 5 levels (mbsolve-tool.cpp:
    310-410): one 5 mm active region with semi-transparent end mirrors of
    power reflectivity 0.8. The reference stores that boundary
    (bc_field_reflectivity) and applies none (every solver keeps the PMC
    boundary); mirror=True applies it instead (bc_field_mirror, opt-in, no
    reference counterpart). The initial E field is random (the scenario's
    density-only constructor); `seed` makes the draw reproducible. A
    shorter `length` with num_gridpoints = 8192 length / 5 mm keeps the
    reference's grid spacing (the records lie within 0.1 mm)."""
    e = mb.E0
    H = mb.qm_operator([0.10103 * e, 0.09677 * e, 0.09720 * e, 0.08129 * e,
                        0.07633 * e],
                       [0.0, 1.2329e-3 * e, -1.3447e-3 * e] + [0.0] * 7)
    # dipole between levels 2 and 3 (upper index (2, 3), column-major)
    u = mb.qm_operator([0.0] * 5, [0.0] * 5 + [-e * 4e-9] + [0.0] * 4)
    scat = [[0.0, 0.4947e12, 0.0974e12, 0.8116e12, 1.0410e12],
            [0.8245e12, 0.0, 0.1358e12, 0.6621e12, 1.1240e12],
            [0.0229e12, 0.0469e12, 0.0, 0.0794e12, 0.0357e12],
            [0.0047e12, 0.0029e12, 0.1252e12, 0.0, 0.2810e12],
            [0.0049e12, 0.0049e12, 0.1101e12, 0.4949e12, 0.0]]
    inj_ull = 1.0 / 1.6e-12
    other = 1.0 / 4.8e-12
    deph = [0.0, inj_ull, inj_ull] + [other] * 7
    qm = mb.qm_description(5.6e21, H, u,
                           mb.qm_lindblad_relaxation(scat, deph))
    ar = _material("AR", qm, 19.35, 0.9, 1300)
    bc = (mb.bc_field_mirror if mirror else mb.bc_field_reflectivity)(0.8,
                                                                      0.8)
    dev = mb.device("tzenov2016", bc)
    dev.add_region(mb.region("Active region", ar, 0, length))
    sce = mb.scenario("basic", num_gridpoints, endtime,
                      mb.qm_operator([0.0, 0.0, 1.0, 0.0, 0.0]))
    if seed is not None:
        sce.set_ic_electric(mb.ic_field_random(seed=seed))
    sce.add_record(mb.record("e0", mb.record.electric, 1, 1, 0.0, 0.0))
    for i in range(1, 6):
        sce.add_record(mb.record("d%d%d" % (i, i), mb.record.density, i, i,
                                 0.0, 0.1e-3))
    return dev, sce


def tzenov2018_cpml(num_gridpoints=8192, endtime=2e-9, seed=None):
    """Colliding-pulse mode locking, absorber between two gain sections
    (mbsolve-tool.cpp:411-478); `seed` as in tzenov2016."""
    qm_gain = mb.qm_desc_2lvl(5e21, 2 * mb.PI * 3.4e12, 2e-9, 1.0 / 10e-12,
                              1.0 / 200e-15, 1.0)
    qm_abs = mb.qm_desc_2lvl(1e21, 2 * mb.PI * 3.4e12, 6e-9, 1.0 / 3e-12,
                             1.0 / 160e-15)
    mat_abs = _material("Absorber", qm_abs, 12.96, 1.0, 500)
    mat_gain = _material("Gain", qm_gain, 12.96, 1.0, 500)
    dev = mb.device("tzenov-cpml")
    dev.add_region(mb.region("Gain R", mat_gain, 0, 0.5e-3))
    dev.add_region(mb.region("Absorber", mat_abs, 0.5e-3, 0.625e-3))
    dev.add_region(mb.region("Gain L", mat_gain, 0.625e-3, 1.125e-3))
    sce = mb.scenario("basic", num_gridpoints, endtime,
                      mb.qm_operator([0.5, 0.5], [0.001]))
    if seed is not None:
        sce.set_ic_electric(mb.ic_field_random(seed=seed))
    sce.add_record(mb.record("inv12", 1e-12))
    sce.add_record(mb.record("e", 1e-12))
    sce.add_record(mb.record("e0", mb.record.electric, 1, 1, 0.0, 0.0))
    sce.add_record(mb.record("h0", mb.record.magnetic, 1, 1, 0.0, 1.373e-7))
    return dev, sce


# ------------------------------------------------- benchmark workloads

DIPOLE = 1e-29  # C m
FWHM = 100e-15
BETA = 2.0 * math.acosh(2.0) / FWHM  # sech(beta t): FWHM of the envelope
LENGTH_2LVL = 150e-6


def sech_area_amplitude(area, dipole=DIPOLE, beta=BETA):
    """Amplitude A of A sech(beta t) sin(w t) with pulse area
    mu A pi / (hbar beta) = area."""
    return area * mb.HBAR * beta / (dipole * math.pi)


def sit_2lvl(num_gridpoints=16384, num_timesteps=100000, area=2 * math.pi,
             detuning=0.0, t2=1e-9, t1=1e-9, length=None, phase=15.0,
             probe_interval=0.0):
    """2-level medium filling the whole device (the plain-method workload:
    16,384 points over 150 um, 100,000 steps at Courant 0.5, transition
    2 pi 2e14 rad/s, dipole 1e-29 C m, density 1e24 m^-3, T1 = T2 = 1 ns,
    ground state, hard sech source at x = 0 of the given area and 100 fs
    FWHM, probe E at the output facet every step)."""
    if length is None:
        length = LENGTH_2LVL * (num_gridpoints - 1) / 16383.0
    w0 = 2 * mb.PI * 2e14 * (1.0 + detuning)
    qm = mb.qm_desc_2lvl(1e24, w0, DIPOLE / mb.E0, 1.0 / t1, 1.0 / t2, -1.0)
    ar = _material("AR_2lvl", qm)
    dev = mb.device("sit-2lvl")
    dev.add_region(mb.region("Active region", ar, 0.0, length))
    t_end = _courant_endtime(num_gridpoints, length, num_timesteps)
    sce = mb.scenario("sit", num_gridpoints, t_end,
                      mb.ic_density_const(mb.qm_operator([1, 0])),
                      mb.ic_field_const(0.0), mb.ic_field_const(0.0))
    sce.add_source(mb.sech_pulse("sech", 0.0, mb.source.hard_source,
                                 sech_area_amplitude(area), 2e14, phase,
                                 BETA))
    sce.add_record(mb.record("e", probe_interval, length))
    return dev, sce


def ensemble_2lvl(num_runs=4096, num_timesteps=50000, seed=0,
                  min_points=2048, max_points=32768):
    """Batched 2-level ensemble: lengths uniform in [min, max] points at the
    plain workload's grid spacing, pulse area uniform in [0.5 pi, 4 pi],
    detuning uniform in +-5 %, T2 log-uniform in [0.1, 10] ps; otherwise the
    plain workload's physics. Returns [(device, scenario)] and the sampled
    parameters."""
    rng = np.random.default_rng(seed)
    n_x = rng.integers(min_points, max_points + 1, size=num_runs)
    area = rng.uniform(0.5 * math.pi, 4 * math.pi, size=num_runs)
    det = rng.uniform(-0.05, 0.05, size=num_runs)
    t2 = np.exp(rng.uniform(math.log(0.1e-12), math.log(10e-12),
                            size=num_runs))
    dx = LENGTH_2LVL / 16383.0
    runs = []
    for i in range(num_runs):
        length = (int(n_x[i]) - 1) * dx
        runs.append(sit_2lvl(int(n_x[i]), num_timesteps, float(area[i]),
                             float(det[i]), float(t2[i]), 1e-9, length))
    params = dict(num_gridpoints=n_x, area=area, detuning=det, t2=t2)
    return runs, params


def random_nlvl(N=6, num_gridpoints=65536, num_timesteps=200000, seed=0,
                length=150e-6, e_seed=1e5):
    """Seeded random N-level medium: Hermitian Hamiltonian with levels
    uniform in 0-50 meV and complex couplings at 1 % of that scale; dipole
    matrix with min(5, N(N-1)/2) nonzero upper entries of magnitude
    1e-29-5e-29 C m; scattering and pure-dephasing rates log-uniform in
    1e9-1e12 1/s; ground state; constant seed field e_seed V/m (the
    reference has no CW source class: source.hpp:129-145 is commented out)
    and a probe at the output facet."""
    rng = np.random.default_rng(seed)
    levels = np.sort(rng.uniform(0, 50e-3, size=N)) * mb.E0
    P = N * (N - 1) // 2
    hoff = (rng.normal(size=P) + 1j * rng.normal(size=P)) * 0.01 * 50e-3 * mb.E0
    doff = np.zeros(P, dtype=complex)
    nz = rng.choice(P, size=min(5, P), replace=False)
    doff[nz] = rng.uniform(1e-29, 5e-29, size=len(nz)) * \
        np.exp(1j * rng.uniform(0, 2 * math.pi, size=len(nz)))
    H = mb.qm_operator(list(levels), list(hoff))
    u = mb.qm_operator([0.0] * N, list(doff))
    scat = np.exp(rng.uniform(math.log(1e9), math.log(1e12), size=(N, N)))
    np.fill_diagonal(scat, 0.0)
    deph = np.exp(rng.uniform(math.log(1e9), math.log(1e12), size=P))
    relax = mb.qm_lindblad_relaxation(scat.tolist(), list(deph))
    qm = mb.qm_description(1e24, H, u, relax)
    ar = _material("AR_%dlvl" % N, qm)
    dev = mb.device("random-%dlvl" % N)
    dev.add_region(mb.region("Active region", ar, 0.0, length))
    t_end = _courant_endtime(num_gridpoints, length, num_timesteps)
    rho = [1.0] + [0.0] * (N - 1)
    sce = mb.scenario("random", num_gridpoints, t_end,
                      mb.ic_density_const(mb.qm_operator(rho)),
                      mb.ic_field_const(e_seed), mb.ic_field_const(0.0))
    sce.add_record(mb.record("e", 0.0, length))
    return dev, sce


def lambda_3lvl(num_gridpoints=1048576, num_timesteps=500000,
                length=None, separation=200e-15, probe=None):
    """3-level Lambda medium: levels 0 and 2 coupled to the upper level 1
    by dipoles; two sech pulses 200 fs apart, the second at a 10 % higher
    carrier frequency; probe at the output facet."""
    if length is None:
        length = LENGTH_2LVL * (num_gridpoints - 1) / 16383.0
    w = 2 * mb.PI * 2e14
    H = mb.qm_operator([0.0, mb.HBAR * w, 0.1 * mb.HBAR * w])
    # (0,1), (0,2), (1,2) in column-major upper order
    u = mb.qm_operator([0, 0, 0], [-DIPOLE, 0.0, -DIPOLE])
    relax = mb.qm_lindblad_relaxation(
        [[0, 1e9, 0], [0, 0, 0], [0, 1e9, 0]], [1e10, 1e10, 1e10])
    qm = mb.qm_description(1e24, H, u, relax)
    ar = _material("AR_Lambda", qm)
    dev = mb.device("lambda-3lvl")
    dev.add_region(mb.region("Active region", ar, 0.0, length))
    t_end = _courant_endtime(num_gridpoints, length, num_timesteps)
    sce = mb.scenario("lambda", num_gridpoints, t_end,
                      mb.ic_density_const(mb.qm_operator([1, 0, 0])),
                      mb.ic_field_const(0.0), mb.ic_field_const(0.0))
    a = sech_area_amplitude(math.pi)
    sce.add_source(mb.sech_pulse("sech1", 0.0, mb.source.soft_source, a,
                                 2e14, 15.0, BETA))
    sce.add_source(mb.sech_pulse("sech2", 0.0, mb.source.soft_source, a,
                                 2.2e14, 15.0 + separation * BETA, BETA))
    sce.add_record(mb.record("e", 0.0, length if probe is None else probe))
    return dev, sce
