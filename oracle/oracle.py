"""ctypes bindings for the CPU oracle (liboracle.so) and the compiled reference
network code (oracle/_ref/libref_<net>.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product library.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DATA = os.path.join(ROOT, "data")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)
NAME = 16


class OrcNet(C.Structure):
    _fields_ = [
        ("nspec", C.c_int), ("nreac", C.c_int), ("neq", C.c_int),
        ("spec", C.c_void_p), ("abund0", _dp), ("mass", _dp), ("charge", _ip),
        ("reac", C.c_void_p), ("prod", C.c_void_p),
        ("alpha", _dp), ("beta", _dp), ("gamma", _dp), ("rtmin", _dp), ("rtmax", _dp),
        ("duplicate", _ip), ("ode_kind", _ip), ("rate_kind", _ip), ("ri", _ip), ("pi", _ip),
        ("iH", C.c_int), ("iH2", C.c_int), ("iHD", C.c_int), ("iCO", C.c_int), ("iC", C.c_int),
        ("iS", C.c_int), ("iCx", C.c_int), ("iO", C.c_int), ("iHe", C.c_int), ("iHx", C.c_int),
        ("iHEx", C.c_int), ("iH2x", C.c_int), ("iH3x", C.c_int), ("iH3Ox", C.c_int),
        ("iHCOx", C.c_int), ("ielect", C.c_int),
    ]


class OrcPhys(C.Structure):
    _fields_ = [("zeta", C.c_double), ("omega", C.c_double), ("grain_radius", C.c_double),
                ("metallicity", C.c_double), ("g2d", C.c_double), ("v_turb", C.c_double),
                ("h2form", C.c_int), ("xlambda_linear", C.c_int)]


class OrcCoolant(C.Structure):
    _fields_ = [("nlev", C.c_int), ("ntemp", C.c_int), ("nlin", C.c_int),
                ("energies", _dp), ("weights", _dp), ("A", _dp), ("B", _dp), ("freq", _dp),
                ("temps", _dp), ("col", _dp), ("line_up", _ip), ("line_lo", _ip)]


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def _load(opt="O2"):
    path = os.path.join(HERE, "liboracle.so" if opt == "O2" else f"liboracle_{opt}.so")
    if not os.path.exists(path):
        raise RuntimeError("oracle not built: run `make -C oracle` (or __graft_entry__.build())")
    lib = C.CDLL(path)
    lib.orc_net_load.restype = C.POINTER(OrcNet)
    lib.orc_net_load.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
    lib.orc_net_free.argtypes = [C.POINTER(OrcNet)]
    lib.orc_net_load_layout.restype = C.c_int
    lib.orc_net_load_layout.argtypes = [C.POINTER(OrcNet), C.c_char_p, C.c_char_p, C.c_int]
    lib.orc_rhs.argtypes = [C.POINTER(OrcNet), _dp, C.c_double, _dp, _dp, _dp]
    lib.orc_jac.argtypes = [C.POINTER(OrcNet), _dp, C.c_double, _dp, _dp]
    lib.orc_jac_xe_const.argtypes = [C.POINTER(OrcNet), _dp, C.c_double, _dp, C.c_double, _dp]
    lib.orc_calculate_abundances.restype = C.c_int
    lib.orc_calculate_abundances.argtypes = [C.POINTER(OrcNet), _dp, _dp, _dp, _dp, C.c_int,
                                             C.c_double, C.c_double, C.c_double, C.c_double,
                                             C.c_int, _lp]
    lib.orc_rates_batched.restype = C.c_int
    lib.orc_rates_batched.argtypes = [C.POINTER(OrcNet), C.POINTER(OrcPhys), C.c_int, C.c_int,
                                      _dp, _dp, _dp, _dp, _dp, _dp, C.c_int]
    lib.orc_rates_cell.restype = C.c_int
    lib.orc_rates_cell.argtypes = [C.POINTER(OrcNet), C.POINTER(OrcPhys), C.c_double, C.c_double,
                                   C.c_int, _dp, _dp, _dp, _dp, _ip]
    for fn in ("orc_h2shield1",):
        getattr(lib, fn).restype = C.c_double
        getattr(lib, fn).argtypes = [C.c_double] * 3
    lib.orc_coshield.restype = C.c_double
    lib.orc_coshield.argtypes = [C.c_double, C.c_double]
    lib.orc_lbar.restype = C.c_double
    lib.orc_lbar.argtypes = [C.c_double, C.c_double]
    lib.orc_scatter.restype = C.c_double
    lib.orc_scatter.argtypes = [C.c_double, C.c_double, C.c_int]
    lib.orc_xlambda.restype = C.c_double
    lib.orc_xlambda.argtypes = [C.c_double, C.c_int]
    lib.orc_h2_formation_rate.restype = C.c_double
    lib.orc_h2_formation_rate.argtypes = [C.c_double] * 4
    lib.orc_coolant_load.restype = C.POINTER(OrcCoolant)
    lib.orc_coolant_load.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_char_p, C.c_int]
    lib.orc_levpop_batched.restype = C.c_int
    lib.orc_levpop_batched.argtypes = [C.POINTER(OrcCoolant), C.c_int, _dp, _dp, _dp, _dp, _dp,
                                       _dp, _dp, C.c_int, C.c_int, C.c_double, C.c_double,
                                       _dp, _dp, _dp, C.c_int]
    lib.orc_gauss_jordan.restype = C.c_int
    lib.orc_gauss_jordan.argtypes = [_dp, C.c_int, _dp]
    lib.orc_solvlevpop.restype = C.c_int
    lib.orc_solvlevpop.argtypes = [C.c_int, _dp, C.c_double, _dp]
    lib.orc_lte.argtypes = [C.POINTER(OrcCoolant), C.c_double, C.c_double, _dp]
    lib.orc_heating.argtypes = [C.POINTER(OrcNet), C.c_int, C.POINTER(OrcPhys), C.c_double,
                                C.c_double, C.c_double, C.c_double, _dp, _dp, _ip, _dp]
    _lp64 = C.POINTER(C.c_longlong)
    lib.orc_uvfield.argtypes = [C.c_int, C.c_int, _ip, _lp64, _dp, _ip, _dp, C.c_int, _dp, _dp, C.c_double,
                                _dp, _dp, _dp, _dp]
    lib.orc_columns.argtypes = [C.c_int, C.c_int, _ip, _lp64, _dp, _ip, _dp, _dp, C.c_int, _ip, C.c_int, _dp]
    lib.orc_tau.argtypes = [C.POINTER(OrcCoolant), C.c_int, C.c_int, _ip, _lp64, _dp, _ip, _dp, _dp, C.c_double, _dp]
    _ucp = C.POINTER(C.c_ubyte)
    lib.orc_thermal_balance.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                        C.c_int, _dp, C.c_int, C.c_int, C.POINTER(_dp), _dp, _dp, _dp, _dp, _dp,
                                        _dp, _dp, _ucp, _lp64]
    lib.orc_level_convergence.argtypes = [C.c_int, C.c_int, _ip, C.POINTER(_dp), C.POINTER(_dp), _dp, C.c_int, _ip,
                                          C.c_int, _ucp, _ucp, _lp64]
    return lib


_LIBS = {}


def lib(opt="O2"):
    """The oracle library: "O2" (default) or "O0" (the same sources built at the
    reference's own C optimisation level, for the CPU baseline)."""
    if opt not in _LIBS:
        _LIBS[opt] = _load(opt)
    return _LIBS[opt]


NETWORKS = {"reduced": 0, "full": 1, "mynetwork": 2}
# (nlev, ntemp) per coolant, input_parameters.F90:120-127
COOLANTS = {"CII": ("12c+.dat", 5, 18), "CI": ("12c.dat", 5, 29), "OI": ("16o.dat", 5, 27),
            "CO": ("12co.dat", 41, 25)}


class Network:
    """Oracle view of one chemical network (species_<name>.d / rates_<name>.d).

    layout "reference": slot layout and electron sum of the reference's
    generated code (data/layout_<name>.d); "file": species-file order with
    charges from the species names."""

    def __init__(self, name, data_dir=DATA, layout="reference", opt="O2"):
        self.name = name
        self.L = lib(opt)
        err = C.create_string_buffer(256)
        sp = os.path.join(data_dir, f"species_{name}.d").encode()
        rp = os.path.join(data_dir, f"rates_{name}.d").encode()
        self.p = self.L.orc_net_load(sp, rp, err, 256)
        if not self.p:
            raise RuntimeError(err.value.decode())
        lay = os.path.join(data_dir, f"layout_{name}.d")
        if layout == "reference" and os.path.exists(lay):
            if self.L.orc_net_load_layout(self.p, lay.encode(), err, 256):
                raise RuntimeError(err.value.decode())
        n = self.p.contents
        self.nspec, self.nreac, self.neq = n.nspec, n.nreac, n.neq
        self.charge = np.ctypeslib.as_array(n.charge, (self.nspec,)).copy()
        self.ode_kind = np.ctypeslib.as_array(n.ode_kind, (self.nreac,)).copy()
        self.rate_kind = np.ctypeslib.as_array(n.rate_kind, (self.nreac,)).copy()
        self.duplicate = np.ctypeslib.as_array(n.duplicate, (self.nreac,)).copy()
        names = (C.c_char * NAME * self.nspec).from_address(n.spec)
        self.species = [bytes(x).split(b"\0")[0].decode() for x in names]
        self.idx = {k: getattr(n, k) for k, _ in OrcNet._fields_[19:]}

    def __del__(self):
        try:
            self.L.orc_net_free(self.p)
        except Exception:
            pass

    def rhs(self, rate, n_H, x):
        rate = np.ascontiguousarray(rate, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        ode = np.zeros(self.neq)
        xe = C.c_double()
        self.L.orc_rhs(self.p, _ptr(rate), n_H, _ptr(x), _ptr(ode), C.byref(xe))
        return ode, xe.value

    def jac(self, rate, n_H, x):
        rate = np.ascontiguousarray(rate, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        J = np.zeros((self.neq, self.neq))
        self.L.orc_jac(self.p, _ptr(rate), n_H, _ptr(x), _ptr(J))
        return J

    def jac_xe_const(self, rate, n_H, x, x_e):
        rate = np.ascontiguousarray(rate, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        J = np.zeros((self.neq, self.neq))
        self.L.orc_jac_xe_const(self.p, _ptr(rate), n_H, _ptr(x), x_e, _ptr(J))
        return J

    def calculate_abundances(self, abundance, rate, density, temperature, reltol=1e-8,
                             abstol=1e-30, start_time=0.0, end_time=1e7, nthreads=0,
                             want_stats=False):
        """Restatement of calculate_abundances_; abundance (npart, nspec) updated copy."""
        ab = np.ascontiguousarray(abundance, dtype=np.float64).copy()
        rate = np.ascontiguousarray(rate, dtype=np.float64)
        dens = np.ascontiguousarray(density, dtype=np.float64)
        temp = np.ascontiguousarray(temperature, dtype=np.float64)
        npart = ab.shape[0]
        stats = np.zeros((npart, 8), dtype=np.int64) if want_stats else None
        st = self.L.orc_calculate_abundances(self.p, _ptr(ab), _ptr(rate), _ptr(dens), _ptr(temp),
                                             npart, reltol, abstol, start_time, end_time, nthreads,
                                             _ptr(stats, _lp) if want_stats else None)
        return (ab, st, stats) if want_stats else (ab, st)

    def rates(self, phys, T, Td, rad_surface, AV, column5, nthreads=0, zeta=None):
        """zeta (ncell,) or None: per-cell ZETA of the cosmic-ray variant
        (calc_reac_rates.F90 of 3dpdr_cr.tgz takes zetacrlocal in place of ZETA)."""
        if zeta is not None:
            out = np.zeros((len(T), self.nreac))
            st = 0
            for c in range(len(T)):
                ph = OrcPhys(float(zeta[c]), phys.omega, phys.grain_radius, phys.metallicity, phys.g2d,
                             phys.v_turb, phys.h2form, phys.xlambda_linear)
                out[c:c + 1], s = self.rates(ph, T[c:c + 1], Td[c:c + 1], rad_surface[c:c + 1], AV[c:c + 1],
                                             column5[c:c + 1], nthreads=1)
                st = st or s
            return out, st
        T = np.ascontiguousarray(T, dtype=np.float64)
        ncell = T.shape[0]
        nrays = rad_surface.shape[1]
        out = np.zeros((ncell, self.nreac))
        args = [np.ascontiguousarray(a, dtype=np.float64) for a in (Td, rad_surface, AV, column5)]
        st = self.L.orc_rates_batched(self.p, C.byref(phys), ncell, nrays, _ptr(T),
                                      *[_ptr(a) for a in args], _ptr(out), nthreads)
        return out, st

    def rates_cell(self, phys, T, Td, rad_surface, AV, column5):
        out = np.zeros(self.nreac)
        nr = np.zeros(6, dtype=np.int32)
        args = [np.ascontiguousarray(a, dtype=np.float64) for a in (rad_surface, AV, column5)]
        st = self.L.orc_rates_cell(self.p, C.byref(phys), T, Td, len(rad_surface),
                                   *[_ptr(a) for a in args], _ptr(out), _ptr(nr, _ip))
        return out, nr, st


def phys(zeta_s=5e-17, omega=0.42, grain_radius=1e-7, metallicity=1.0, g2d=100.0,
         v_turb_kms=1.0, h2form=1, xlambda_linear=0):
    return OrcPhys(zeta_s / 1.3e-17, omega, grain_radius, metallicity, g2d, v_turb_kms * 1e5,
                   h2form, xlambda_linear)


class Coolant:
    def __init__(self, key, data_dir=DATA):
        fname, nlev, ntemp = COOLANTS[key]
        err = C.create_string_buffer(256)
        self.p = lib().orc_coolant_load(os.path.join(data_dir, fname).encode(), nlev, ntemp, err, 256)
        if not self.p:
            raise RuntimeError(err.value.decode())
        c = self.p.contents
        self.nlev, self.ntemp, self.nlin = c.nlev, c.ntemp, c.nlin
        nl = self.nlev
        self.energies = np.ctypeslib.as_array(c.energies, (nl,)).copy()
        self.weights = np.ctypeslib.as_array(c.weights, (nl,)).copy()
        self.A = np.ctypeslib.as_array(c.A, (nl, nl)).copy()
        self.B = np.ctypeslib.as_array(c.B, (nl, nl)).copy()
        self.freq = np.ctypeslib.as_array(c.freq, (nl, nl)).copy()
        self.temps = np.ctypeslib.as_array(c.temps, (7, self.ntemp)).copy()
        self.col = np.ctypeslib.as_array(c.col, (7, nl, nl, self.ntemp)).copy()
        self.line_up = np.ctypeslib.as_array(c.line_up, (self.nlin,)).copy()
        self.line_lo = np.ctypeslib.as_array(c.line_lo, (self.nlin,)).copy()

    def optical_depths(self, r, pop, T, v_turb):
        """Line optical depths along the rays of workloads.rays(): (ncell, nlin, nrays)."""
        ep, off, xyz, gp = _rays_arrays(r)
        pop = np.ascontiguousarray(pop, dtype=np.float64)
        T = np.ascontiguousarray(T, dtype=np.float64)
        out = np.zeros(r["ncell"] * self.nlin * r["nrays"])
        lib().orc_tau(self.p, r["ncell"], r["nrays"], _ptr(ep, _ip), off.ctypes.data_as(C.POINTER(C.c_longlong)),
                      _ptr(xyz), _ptr(gp, _ip), _ptr(pop), _ptr(T), v_turb, _ptr(out))
        return out.reshape(r["ncell"], self.nlin, r["nrays"])

    def lte(self, T, density):
        pop = np.zeros(self.nlev)
        lib().orc_lte(self.p, T, density, _ptr(pop))
        return pop

    def levpop(self, density, T, Tdust, partner5, coolant_density, s_pop, tau, pseudo1d=0,
               metallicity=1.0, g2d=100.0, nthreads=0):
        ncell = len(density)
        nrays = tau.shape[-1]
        pop = np.zeros((ncell, self.nlev))
        cool = np.zeros(ncell)
        line = np.zeros((ncell, self.nlev, self.nlev))
        arrs = [np.ascontiguousarray(a, dtype=np.float64)
                for a in (density, T, Tdust, partner5, coolant_density, s_pop, tau)]
        st = lib().orc_levpop_batched(self.p, ncell, *[_ptr(a) for a in arrs], nrays, pseudo1d,
                                      metallicity, g2d, _ptr(pop), _ptr(cool), _ptr(line), nthreads)
        return pop, cool, line, st


class RefNetwork:
    """The reference's generated f()/Jac() compiled from its own sources (oracle/_ref)."""

    def __init__(self, name):
        path = os.path.join(HERE, "_ref", f"libref_{name}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.lib.ref_rhs.restype = C.c_double
        self.lib.ref_rhs.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double]
        self.lib.ref_jac.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double]

    def rhs(self, neq, rate, n_H, x, T=100.0):
        rate = np.ascontiguousarray(rate, dtype=np.float64).copy()
        x = np.ascontiguousarray(x, dtype=np.float64)
        ode = np.zeros(neq)
        xe = self.lib.ref_rhs(neq, _ptr(x), _ptr(ode), _ptr(rate), n_H, T)
        return ode, xe

    def jac(self, neq, rate, n_H, x, x_e, T=100.0):
        rate = np.ascontiguousarray(rate, dtype=np.float64).copy()
        x = np.ascontiguousarray(x, dtype=np.float64)
        J = np.zeros((neq, neq))  # column-major from the reference: J[j, i]
        self.lib.ref_jac(neq, _ptr(x), _ptr(J), _ptr(rate), n_H, T, x_e)
        return J.T.copy()


def _rays_arrays(r):
    return (np.ascontiguousarray(r["epray"], dtype=np.int32), np.ascontiguousarray(r["offset"], dtype=np.int64),
            np.ascontiguousarray(r["xyz"], dtype=np.float64), np.ascontiguousarray(r["gridpoint"], dtype=np.int32))


def uvfield(r, field=0, G=(10.0, 0.0, 0.0), metallicity=1.0):
    """CALC_UVFIELD over the rays of workloads.rays(): (columndensity, AV, rad_surface, UVfield)."""
    ep, off, xyz, gp = _rays_arrays(r)
    n, nr = r["ncell"], r["nrays"]
    col, av, rad, uv = np.zeros(n * nr), np.zeros(n * nr), np.zeros(n * nr), np.zeros(n)
    g = np.ascontiguousarray(G, dtype=np.float64)
    vec = np.ascontiguousarray(r["vectors"], dtype=np.float64)
    rho = np.ascontiguousarray(r["rho"], dtype=np.float64)
    lib().orc_uvfield(n, nr, _ptr(ep, _ip), off.ctypes.data_as(C.POINTER(C.c_longlong)), _ptr(xyz), _ptr(gp, _ip),
                      _ptr(rho), field, _ptr(g), _ptr(vec), metallicity, _ptr(col), _ptr(av), _ptr(rad), _ptr(uv))
    return col.reshape(n, nr), av.reshape(n, nr), rad.reshape(n, nr), uv


def columns(r, species=None):
    """calc_columndens over the rays of workloads.rays(): (ncell, nrays, nsel)."""
    ep, off, xyz, gp = _rays_arrays(r)
    n, nr = r["ncell"], r["nrays"]
    ab = np.ascontiguousarray(r["abundance"], dtype=np.float64)
    nspec = ab.shape[1]
    sp = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
    nsel = nspec if sp is None else len(sp)
    out = np.zeros(n * nr * nsel)
    rho = np.ascontiguousarray(r["rho"], dtype=np.float64)
    lib().orc_columns(n, nr, _ptr(ep, _ip), off.ctypes.data_as(C.POINTER(C.c_longlong)), _ptr(xyz), _ptr(gp, _ip),
                      _ptr(rho), _ptr(ab), nspec, _ptr(sp, _ip) if sp is not None else None, nsel, _ptr(out))
    return out.reshape(n, nr, nsel)


def thermal_balance(state, heating_total, cooling, level_conv, first_time, Tmin=2.7, Tmax=30000.0, Fcrit=0.005,
                    Tdiff=0.01, temp_fix=True):
    """3DPDR.F90:928-1050 on numpy state (dict of T, Tprev, Tlow, Thigh, Fmean,
    Fratio float64 arrays and flags uint8), updated in place; returns
    (total cooling, number converged)."""
    n = state["T"].shape[0]
    heat = np.ascontiguousarray(heating_total, dtype=np.float64)
    cools = [np.ascontiguousarray(c, dtype=np.float64) for c in cooling]
    cp = (_dp * len(cools))(*[_ptr(c) for c in cools])
    for k in ("T", "Tprev", "Tlow", "Thigh", "Fmean", "Fratio"):
        assert state[k].dtype == np.float64 and state[k].flags.c_contiguous
    assert state["flags"].dtype == np.uint8
    total = np.zeros(n)
    nconv = C.c_longlong(0)
    lib().orc_thermal_balance(n, Tmin, Tmax, Fcrit, Tdiff, 1 if temp_fix else 0, int(bool(level_conv)),
                              int(bool(first_time)), _ptr(heat), 1, len(cools), cp,
                              *[_ptr(state[k]) for k in ("T", "Tprev", "Tlow", "Thigh", "Fmean", "Fratio")],
                              _ptr(total), state["flags"].ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(nconv))
    return total, nconv.value


def level_convergence(solutions, pops, abundance, species, flags, thermal_balance=True):
    """3DPDR.F90:1084-1229: pops (list of (ncell, nlev) float64) overwritten with
    solutions, flags updated; returns (coolant_conv bits, counts)."""
    k = len(solutions)
    n = solutions[0].shape[0]
    sols = [np.ascontiguousarray(s, dtype=np.float64) for s in solutions]
    for p in pops:
        assert p.dtype == np.float64 and p.flags.c_contiguous
    ab = np.ascontiguousarray(abundance, dtype=np.float64)
    nlev = (C.c_int * k)(*[s.shape[1] for s in sols])
    sp = (C.c_int * k)(*[int(x) for x in species])
    cconv = np.zeros(n, dtype=np.uint8)
    counts = np.zeros(1 + k, dtype=np.int64)
    lib().orc_level_convergence(n, k, nlev, (_dp * k)(*[_ptr(s) for s in sols]), (_dp * k)(*[_ptr(p) for p in pops]),
                                _ptr(ab), ab.shape[1], sp, int(bool(thermal_balance)),
                                flags.ctypes.data_as(C.POINTER(C.c_ubyte)), cconv.ctypes.data_as(C.POINTER(C.c_ubyte)),
                                counts.ctypes.data_as(C.POINTER(C.c_longlong)))
    return cconv, counts
