"""Python mirror of mbsolve's public API (the SWIG module ``mbsolve.lib``).

Same class names, constructor arguments, defaults and error behaviour as
the reference's C++ classes, so that scripts written for ``mbsolve.lib``
(e.g. tools/python/ziolkowski1995.py) run by changing the import and the
solver name. Each class cites the reference header it mirrors.

The objects are plain Python; :func:`to_pod` flattens a device/scenario
pair into the C structs of include/mbsolve_gb300.h for the GPU engine.
"""
import bisect
import math

import numpy as np

from . import capi_types as T

# types.hpp:36-73
HBAR = 1.05457266e-34
PI = math.atan(1.0) * 4.0
MU0 = PI * 4e-7
EPS0 = 8.854187817e-12
E0 = 1.60217733e-19
KB = 1.38064852e-23


class qm_operator:
    """qm_description.hpp:38-87: main diagonal (real) and the upper
    off-diagonal triangle in column-major order (complex)."""

    def __init__(self, main_diagonal, off_diagonal=()):
        self._main = [float(x) for x in main_diagonal]
        self._off = [complex(x) for x in off_diagonal]

    def get_num_levels(self):
        return len(self._main)

    def get_main_diagonal(self):
        return list(self._main)

    def get_off_diagonal(self):
        return list(self._off)


class qm_superop:
    """qm_description.hpp:93-138: the base superoperator acts as zero."""

    def __init__(self, num_levels):
        self._n = int(num_levels)

    def get_num_levels(self):
        return self._n

    def action(self, arg):
        return qm_operator([0.0] * self._n)

    def __call__(self, arg):
        return self.action(arg)


class qm_lindblad_relaxation(qm_superop):
    """qm_description.hpp:144-253. The constructor replaces the diagonal of
    the scattering matrix with the negative inverse lifetimes and folds the
    lifetimes into the dephasing rates, exactly as the reference does."""

    def __init__(self, scattering_rates, pure_deph_rates):
        s = [[float(x) for x in row] for row in scattering_rates]
        n = len(s)
        super().__init__(n)
        for m in range(n):
            inv = 0.0
            for j in range(n):
                if j != m:
                    inv += s[j][m]
            s[m][m] = -inv
        deph = [float(x) for x in pure_deph_rates]
        idx = 0
        for nn in range(n):
            for m in range(nn):
                d = -abs(deph[idx])
                d -= 0.5 * (abs(s[m][m]) + abs(s[nn][nn]))
                deph[idx] = d
                idx += 1
        self._s = s
        self._d = deph

    def action(self, arg):
        main = arg.get_main_diagonal()
        n = self._n
        pops = [sum(self._s[m][k] * main[k] for k in range(n))
                for m in range(n)]
        coh = [c * self._d[i] for i, c in enumerate(arg.get_off_diagonal())]
        return qm_operator(pops, coh)

    def get_scattering_rates(self):
        return [list(r) for r in self._s]

    def get_dephasing_rates(self):
        return list(self._d)


class qm_description:
    """qm_description.hpp:259-332."""

    def __init__(self, carrier_density, hamiltonian, dipole_operator,
                 relaxation_superop):
        self._n = hamiltonian.get_num_levels()
        self._dens = float(carrier_density)
        self._h = hamiltonian
        self._u = dipole_operator
        self._r = relaxation_superop

    def get_num_levels(self):
        return self._n

    def get_carrier_density(self):
        return self._dens

    def get_hamiltonian(self):
        return self._h

    def get_dipole_operator(self):
        return self._u

    def get_relaxation_superop(self):
        return self._r


class qm_desc_2lvl(qm_description):
    """qm_description.hpp:338-432: H = hbar/2 diag(-w0, w0), dipole
    off-diagonal -e*d, relaxation towards the equilibrium inversion."""

    def __init__(self, carrier_density, transition_freq, dipole_moment,
                 scattering_rate, dephasing_rate, equilibrium_inversion=-1.0):
        w = equilibrium_inversion
        super().__init__(
            carrier_density,
            qm_operator([-HBAR * transition_freq / 2,
                         +HBAR * transition_freq / 2]),
            qm_operator([0, 0], [-E0 * dipole_moment]),
            qm_lindblad_relaxation(
                [[0, scattering_rate * 0.5 * (1 - w)],
                 [scattering_rate * 0.5 * (1 + w), 0]],
                [dephasing_rate - 0.5 * scattering_rate]))
        self._tf = transition_freq
        self._dm = dipole_moment
        self._sr = scattering_rate
        self._dr = dephasing_rate
        self._ei = w

    def get_transition_freq(self):
        return self._tf

    def get_dipole_moment(self):
        return self._dm

    def get_scattering_rate(self):
        return self._sr

    def get_dephasing_rate(self):
        return self._dr

    def get_equilibrium_inversion(self):
        return self._ei


class material:
    """material.hpp:38-130 with its global library (material.cpp:26-47)."""

    _library = {}

    def __init__(self, id, qm=None, rel_permittivity=1.0, overlap_factor=1.0,
                 losses=0.0, rel_permeability=1.0):
        self._id = id
        self._qm = qm
        self._eps = float(rel_permittivity)
        self._overlap = float(overlap_factor)
        self._losses = float(losses)
        self._mu = float(rel_permeability)

    def get_id(self):
        return self._id

    def get_qm(self):
        return self._qm

    def get_rel_permittivity(self):
        return self._eps

    def get_rel_permeability(self):
        return self._mu

    def get_losses(self):
        return self._losses

    def get_overlap_factor(self):
        return self._overlap

    @staticmethod
    def add_to_library(mat):
        if mat.get_id() in material._library:
            raise RuntimeError("Material already available in library.")
        material._library[mat.get_id()] = mat

    @staticmethod
    def get_from_library(id):
        if id not in material._library:
            raise RuntimeError("Material not available in library.")
        return material._library[id]

    @staticmethod
    def clear_library():
        """Not in the reference (its library lives until exit); lets test
        suites start from an empty library."""
        material._library.clear()


class bc_field:
    """device.hpp:38-48."""


class bc_field_reflectivity(bc_field):
    """device.hpp:50-79. Stored, but (as in every reference solver) not
    applied: the time loop uses the PMC boundary H[0] = H[N] = 0."""

    def __init__(self, refl_left=1.0, refl_right=1.0):
        self._l = refl_left
        self._r = refl_right

    def get_refl_left(self):
        return self._l

    def get_refl_right(self):
        return self._r


class bc_field_mirror(bc_field_reflectivity):
    """Not in the reference: semi-transparent mirrors of power reflectivity
    refl_left and refl_right at the device ends, applied by the gpu-fdtd
    solvers (MBG_BC_MIRROR: H beyond each end tied to the end point's E as
    an impedance wall with E-field reflection coefficient sqrt(refl);
    1 is the reference's PMC boundary, 0 absorbs). The reference's own
    bc_field_reflectivity stays stored and unapplied, as in its solvers."""

    def __init__(self, refl_left=1.0, refl_right=1.0):
        bc_field_reflectivity.__init__(self, refl_left, refl_right)


class region:
    """device.hpp:82-150."""

    def __init__(self, name, mat, x_start, x_end):
        self._name = name
        self._mat = mat
        self._x0 = float(x_start)
        self._x1 = float(x_end)

    def get_name(self):
        return self._name

    def get_length(self):
        return self._x1 - self._x0

    def get_x_start(self):
        return self._x0

    def get_x_end(self):
        return self._x1

    def get_material(self):
        return self._mat


class device:
    """device.hpp:152-216, device.cpp:26-90."""

    def __init__(self, name, field_boundary=None):
        self._name = name
        self._regions = []
        self._used = []  # sorted material ids (std::set<std::string>)
        self._bc = field_boundary if field_boundary is not None \
            else bc_field_reflectivity(1.0, 1.0)

    def add_region(self, reg):
        self._regions.append(reg)
        mid = reg.get_material().get_id()
        i = bisect.bisect_left(self._used, mid)
        if i == len(self._used) or self._used[i] != mid:
            self._used.insert(i, mid)

    def get_regions(self):
        return list(self._regions)

    def get_used_materials(self):
        return list(self._used)

    def get_name(self):
        return self._name

    def get_length(self):
        total = 0.0
        for r in self._regions:
            total += r.get_length()
        return total

    def get_minimum_permittivity(self):
        m = 1e42
        for r in self._regions:
            e = r.get_material().get_rel_permittivity()
            if e < m:
                m = e
        return m

    def get_bc_field(self):
        return self._bc

    def set_bc_field(self, bc):
        self._bc = bc


class ic_density:
    """scenario.hpp:40-47."""

    def initialize(self, x):
        raise NotImplementedError


class ic_density_const(ic_density):
    """scenario.hpp:54-78."""

    def __init__(self, rho):
        self._rho = rho

    def initialize(self, x):
        return self._rho


class ic_field:
    """scenario.hpp:85-92."""

    def initialize(self, x):
        raise NotImplementedError


class ic_field_const(ic_field):
    """scenario.hpp:99-117."""

    def __init__(self, field_value):
        self._v = float(field_value)

    def initialize(self, x):
        return self._v


class ic_field_random(ic_field):
    """scenario.hpp:125-157: normal(mean, stddev) * amplitude per grid
    point. The reference seeds from std::random_device (nondeterministic);
    here `seed` (default None = OS entropy) makes a run reproducible."""

    def __init__(self, mean=0.0, stddev=1.0, amplitude=1e-15, seed=None):
        self._mean = mean
        self._std = stddev
        self._amp = amplitude
        self._rng = np.random.default_rng(seed)
        self._cache = {}

    def initialize(self, x):
        return float(self._rng.normal(self._mean, self._std) * self._amp)

    def values(self, n):
        """One draw per grid point; the same draw for every solver that
        reads this initial condition (so that two solvers can be compared)."""
        if n not in self._cache:
            self._cache[n] = self._rng.normal(self._mean, self._std,
                                              size=n) * self._amp
        return self._cache[n]


class source:
    """source.hpp:35-127."""

    hard_source = T.MBG_SOURCE_HARD
    soft_source = T.MBG_SOURCE_SOFT

    class type:
        hard_source = T.MBG_SOURCE_HARD
        soft_source = T.MBG_SOURCE_SOFT

    def __init__(self, name, position, source_type, ampl, freq, phase=0.0):
        self._name = name
        self._pos = float(position)
        self._type = int(source_type)
        self._ampl = float(ampl)
        self._freq = float(freq)
        self._phase = float(phase)

    def calc_value(self, t):
        return 0.0

    def get_value(self, t, current_value=0.0):
        return self._ampl * self.calc_value(t)

    def get_position(self):
        return self._pos

    def get_type(self):
        return self._type

    def _pod_shape(self):
        return T.MBG_SHAPE_TABLE, 0.0, 0.0


class sech_pulse(source):
    """source.hpp:147-196: A sech(beta t - phase) sin(2 pi f t - phase_sin)."""

    def __init__(self, name, position, source_type, ampl, freq, phase, beta,
                 phase_sin=0.0):
        super().__init__(name, position, source_type, ampl, freq, phase)
        self._beta = float(beta)
        self._phase_sin = float(phase_sin)

    def calc_value(self, t):
        return 1 / math.cosh(self._beta * t - self._phase) * \
            math.sin(2 * PI * self._freq * t - self._phase_sin)

    def _pod_shape(self):
        return T.MBG_SHAPE_SECH, self._beta, self._phase_sin


class gaussian_pulse(source):
    """source.hpp:222-261: A exp(-(t - phase)^2/tau^2) sin(2 pi f t)."""

    def __init__(self, name, position, source_type, ampl, freq, phase, tau):
        super().__init__(name, position, source_type, ampl, freq, phase)
        self._tau = float(tau)

    def calc_value(self, t):
        return math.exp(-(t - self._phase) ** 2 / (self._tau ** 2)) * \
            math.sin(2 * PI * self._freq * t)

    def _pod_shape(self):
        return T.MBG_SHAPE_GAUSSIAN, self._tau, 0.0


class record:
    """record.hpp:37-140, record.cpp:27-69. Either record(name, interval,
    position) with the type deduced from the first letter of the name, or
    record(name, type, row_idx, col_idx, interval, position) with one-based
    density indices."""

    electric = T.MBG_RECORD_ELECTRIC
    polar_dt = T.MBG_RECORD_POLAR_DT
    magnetic = T.MBG_RECORD_MAGNETIC
    density = T.MBG_RECORD_DENSITY
    inversion = T.MBG_RECORD_INVERSION

    class type:
        electric = T.MBG_RECORD_ELECTRIC
        polar_dt = T.MBG_RECORD_POLAR_DT
        magnetic = T.MBG_RECORD_MAGNETIC
        density = T.MBG_RECORD_DENSITY
        inversion = T.MBG_RECORD_INVERSION

    _letters = {"e": T.MBG_RECORD_ELECTRIC, "p": T.MBG_RECORD_POLAR_DT,
                "h": T.MBG_RECORD_MAGNETIC, "d": T.MBG_RECORD_DENSITY,
                "i": T.MBG_RECORD_INVERSION}

    def __init__(self, name, *args):
        self._name = name
        if len(args) >= 3:
            rtype, row_idx, col_idx = args[0], args[1], args[2]
            self._interval = float(args[3]) if len(args) > 3 else 0.0
            self._position = float(args[4]) if len(args) > 4 else -1.0
            self._type = int(rtype)
            self._row = int(row_idx) - 1
            self._col = int(col_idx) - 1
        else:
            self._interval = float(args[0]) if len(args) > 0 else 0.0
            self._position = float(args[1]) if len(args) > 1 else -1.0
            if not name or name[0] not in record._letters:
                raise RuntimeError("Unknown record type")
            self._type = record._letters[name[0]]
            # the reference leaves row/col uninitialised here; they are only
            # read for density records
            self._row = 0
            self._col = 0
        self._complex = (self._type == T.MBG_RECORD_DENSITY) and \
            (self._row != self._col)

    def get_name(self):
        return self._name

    def get_type(self):
        return self._type

    def get_col(self):
        return self._col

    def get_row(self):
        return self._row

    def get_position(self):
        return self._position

    def get_interval(self):
        return self._interval

    def is_complex(self):
        return self._complex


class coherence_record(record):
    """Not in the reference: a density record of an off-diagonal entry
    rho[row][col] (one-based indices, row != col) that records its value,
    real and imaginary part. The reference's record of the same entry stays
    zero (solver_cpu_fdtd.tpp:314-318), and so does this package's."""

    def __init__(self, name, row_idx, col_idx, interval=0.0, position=-1.0):
        if int(row_idx) == int(col_idx):
            raise RuntimeError("coherence record needs row != col")
        record.__init__(self, name, record.density, row_idx, col_idx,
                        interval, position)


class result:
    """result.hpp:37-120: row-major [rows x cols] real and imaginary data."""

    def __init__(self, name, cols, rows, is_complex=False, real=None,
                 imag=None):
        self._name = name
        self._cols = int(cols)
        self._rows = int(rows)
        self._complex = bool(is_complex)
        n = self._cols * self._rows
        self._real = np.zeros(n) if real is None else np.asarray(real)
        self._imag = np.zeros(n) if imag is None else np.asarray(imag)

    def get_name(self):
        return self._name

    def get_count(self):
        return self._cols * self._rows

    def get_cols(self):
        return self._cols

    def get_rows(self):
        return self._rows

    def is_complex(self):
        return self._complex

    def get_data_real(self):
        return self._real

    def get_data_imag(self):
        return self._imag

    def get_data_complex(self):
        return self._real + 1j * self._imag

    def as_array(self):
        """[rows, cols] view of the real part (numpy convenience)."""
        return self._real.reshape(self._rows, self._cols)


class scenario:
    """scenario.hpp:164-335, scenario.cpp:26-120. Two constructors as in the
    reference: scenario(name, n_x, t_end, rho_init: qm_operator,
    num_timesteps=2) (random E initial condition) and scenario(name, n_x,
    t_end, density_init, electric_init=ic_field_random(),
    magnetic_init=ic_field_const(0), num_timesteps=2)."""

    def __init__(self, name, num_gridpoints, endtime, init, *args):
        self._name = name
        self._nx = int(num_gridpoints)
        self._endtime = float(endtime)
        self._records = []
        self._sources = []
        self._dt = 0.0
        self._dx = 0.0
        if isinstance(init, qm_operator):
            self._dens = ic_density_const(init)
            self._e = ic_field_random()
            self._h = ic_field_const(0)
            self._nt = int(args[0]) if args else 2
        else:
            self._dens = init
            self._e = args[0] if len(args) > 0 else ic_field_random()
            self._h = args[1] if len(args) > 1 else ic_field_const(0)
            self._nt = int(args[2]) if len(args) > 2 else 2

    def add_record(self, rec):
        self._records.append(rec)

    def get_records(self):
        return list(self._records)

    def add_source(self, src):
        self._sources.append(src)

    def get_sources(self):
        return list(self._sources)

    def get_name(self):
        return self._name

    def get_num_timesteps(self):
        return self._nt

    def set_num_timesteps(self, v):
        self._nt = int(v)

    def get_num_gridpoints(self):
        return self._nx

    def set_num_gridpoints(self, v):
        self._nx = int(v)

    def get_timestep_size(self):
        return self._dt

    def set_timestep_size(self, v):
        self._dt = float(v)

    def get_gridpoint_size(self):
        return self._dx

    def set_gridpoint_size(self, v):
        self._dx = float(v)

    def get_endtime(self):
        return self._endtime

    def set_endtime(self, v):
        self._endtime = float(v)

    def get_ic_density(self):
        return self._dens

    def set_ic_density(self, d):
        self._dens = d

    def get_ic_electric(self):
        return self._e

    def set_ic_electric(self, e):
        self._e = e

    def get_ic_magnetic(self):
        return self._h

    def set_ic_magnetic(self, h):
        self._h = h


class solver:
    """solver.hpp:42-142, solver.cpp:26-84: a name -> bootstrap factory."""

    _bootstraps = {}

    def __init__(self, name, dev, scen):
        self._name = name
        self._device = dev
        self._scenario = scen
        self._results = []

    @staticmethod
    def get_avail_solvers():
        return sorted(solver._bootstraps)

    @staticmethod
    def register_bootstrap(name, bootstrap):
        if name in solver._bootstraps:
            raise RuntimeError("Solver already registered.")
        solver._bootstraps[name] = bootstrap

    @staticmethod
    def register_solver(cls, name):
        solver.register_bootstrap(name, lambda dev, scen: cls(dev, scen,
                                                              name))

    @staticmethod
    def create_instance(name, dev, scen):
        if name not in solver._bootstraps:
            raise RuntimeError("Unknown solver " + name)
        return solver._bootstraps[name](dev, scen)

    def get_name(self):
        return self._name

    def get_scenario(self):
        return self._scenario

    def get_device(self):
        return self._device

    def run(self):
        raise NotImplementedError

    def get_results(self):
        return list(self._results)


# ------------------------------------------------------------ flattening

def _op_arrays(bundle, op, n, full=True):
    """Main diagonal and off-diagonal (re, im) arrays of an operator. With
    `full`, the off-diagonal triangle is padded with zeros (or cut) to
    exactly n(n-1)/2 entries: the reference fills a zero matrix from as many
    entries as the operator holds (coherence_vector_representation.hpp:
    99-130)."""
    main = list(op.get_main_diagonal())[:n]
    main += [0.0] * (n - len(main))
    off = list(op.get_off_diagonal())
    if full:
        p = n * (n - 1) // 2
        off = (off + [0j] * p)[:p]
    flat = []
    for c in off:
        flat += [c.real, c.imag]
    return bundle.hold(T.dbuf(main)), bundle.hold(T.dbuf(flat))


def _qm_pod(bundle, qm):
    n = qm.get_num_levels()
    q = T.mbg_qm()
    q.num_levels = n
    q.carrier_density = qm.get_carrier_density()
    q.h_diag, q.h_off = _op_arrays(bundle, qm.get_hamiltonian(), n)
    q.mu_diag, q.mu_off = _op_arrays(bundle, qm.get_dipole_operator(), n)
    r = qm.get_relaxation_superop()
    if isinstance(r, qm_lindblad_relaxation):
        q.relax_kind = T.MBG_RELAX_LINDBLAD
        s = r.get_scattering_rates()
        q.scattering = bundle.hold(T.dbuf([x for row in s for x in row]))
        q.dephasing = bundle.hold(T.dbuf(r.get_dephasing_rates()))
    elif type(r) is qm_superop or r is None:
        q.relax_kind = T.MBG_RELAX_NONE
        q.scattering = bundle.hold(T.dbuf([0.0] * (n * n)))
        q.dephasing = bundle.hold(T.dbuf([0.0] * max(1, n * (n - 1) // 2)))
    else:
        raise RuntimeError("Unsupported superoperator!")
    return bundle.hold(q)


def to_pod(dev, scen, bundle=None):
    """Flatten (device, scenario) into mbg_device / mbg_scenario structs.

    Materials are listed in device.get_used_materials() order (sorted ids,
    the order of the reference's std::set) and looked up in the material
    library as the reference's solvers do (solver_cpu_fdtd.tpp:76-89)."""
    b = bundle or T.PodBundle()
    used = dev.get_used_materials()
    mats = (T.mbg_material * max(1, len(used)))()
    b.hold(mats)
    index = {}
    for i, mid in enumerate(used):
        m = material.get_from_library(mid)
        mats[i].rel_permittivity = m.get_rel_permittivity()
        mats[i].rel_permeability = m.get_rel_permeability()
        mats[i].overlap_factor = m.get_overlap_factor()
        mats[i].losses = m.get_losses()
        if m.get_qm() is not None:
            import ctypes
            mats[i].qm = ctypes.pointer(_qm_pod(b, m.get_qm()))
        index[mid] = i
    regs = dev.get_regions()
    rarr = (T.mbg_region * max(1, len(regs)))()
    b.hold(rarr)
    for i, r in enumerate(regs):
        rarr[i].material = index[r.get_material().get_id()]
        rarr[i].x_start = r.get_x_start()
        rarr[i].x_end = r.get_x_end()
    d = T.mbg_device()
    d.num_materials = len(used)
    d.materials = mats
    d.num_regions = len(regs)
    d.regions = rarr
    bc = dev.get_bc_field()
    if isinstance(bc, bc_field_mirror):
        d.bc_kind = T.MBG_BC_MIRROR
        d.refl_left = bc.get_refl_left()
        d.refl_right = bc.get_refl_right()
    else:
        d.bc_kind = T.MBG_BC_PMC
        d.refl_left = d.refl_right = 1.0
    b.device = b.hold(d)

    s = T.mbg_scenario()
    nx = scen.get_num_gridpoints()
    s.num_gridpoints = nx
    s.endtime = scen.get_endtime()
    s.num_timesteps = scen.get_num_timesteps()
    icd = scen.get_ic_density()
    if icd is not None:
        rho = icd.initialize(0.0)
        n = rho.get_num_levels()
        s.rho_levels = n
        s.rho_num_off = len(rho.get_off_diagonal())
        s.rho_diag, s.rho_off = _op_arrays(b, rho, n, full=False)
    for which in ("e", "h"):
        ic = scen.get_ic_electric() if which == "e" else \
            scen.get_ic_magnetic()
        if isinstance(ic, ic_field_const):
            kind, val, vals = T.MBG_FIELD_IC_CONST, ic.initialize(0.0), None
        elif isinstance(ic, ic_field_random):
            kind, val = T.MBG_FIELD_IC_VALUES, 0.0
            vals = b.hold(T.dbuf(ic.values(nx)))
        else:
            # any other initial condition: sample it at the grid points,
            # which the solver sets up before calling initialize(x)
            dx = scen.get_gridpoint_size()
            kind, val = T.MBG_FIELD_IC_VALUES, 0.0
            vals = b.hold(T.dbuf([ic.initialize(i * dx) for i in range(nx)]))
        if which == "e":
            s.e_init_kind, s.e_init_value = kind, val
            if vals is not None:
                s.e_init_values = vals
        else:
            s.h_init_kind, s.h_init_value = kind, val
            if vals is not None:
                s.h_init_values = vals
    srcs = scen.get_sources()
    sarr = (T.mbg_source * max(1, len(srcs)))()
    b.hold(sarr)
    for i, so in enumerate(srcs):
        shape, bt, ps = so._pod_shape()
        sarr[i].type = so.get_type()
        sarr[i].shape = shape
        sarr[i].position = so.get_position()
        sarr[i].ampl = so._ampl
        sarr[i].freq = so._freq
        sarr[i].phase = so._phase
        sarr[i].beta_or_tau = bt
        sarr[i].phase_sin = ps
        if shape == T.MBG_SHAPE_TABLE:
            tab = getattr(so, "_table_cache", None)
            if tab is None:
                raise RuntimeError(
                    "custom source: call tabulate(source, n_t, dt) first")
            sarr[i].table = b.hold(T.dbuf(tab))
            sarr[i].table_len = len(tab)
    s.num_sources = len(srcs)
    s.sources = sarr
    recs = scen.get_records()
    rarr2 = (T.mbg_record * max(1, len(recs)))()
    b.hold(rarr2)
    for i, r in enumerate(recs):
        rarr2[i].type = r.get_type()
        rarr2[i].row = max(0, r.get_row())
        rarr2[i].col = max(0, r.get_col())
        rarr2[i].interval = r.get_interval()
        rarr2[i].position = r.get_position()
        rarr2[i].is_complex = int(r.is_complex())
        rarr2[i].coherence = int(isinstance(r, coherence_record))
    s.num_records = len(recs)
    s.records = rarr2
    b.scenario = b.hold(s)
    return b


def tabulate(src, n_t, dt):
    """Precompute a custom source's values get_value(j*dt), j < n_t (what
    solver_cpu_fdtd.tpp:185-202 does for every source)."""
    src._table_cache = [src.get_value(j * dt) for j in range(n_t)]
    return src._table_cache
