"""Reader of the reference's runtime.dat thermo tables, unchanged on disk.

Restates Setup::ReadSpecies / Setup::ReadThermal (src/read_ini/src/thermal.cpp:6-178): the NASA-9
file gives 3 temperature ranges of 7 a-coefficients and 2 b-coefficients per species, the JANAF /
NASA-7 file 2 ranges of 7 coefficients; the molar mass that follows the selected table is the
species' Wi (g/mol, converted to kg/mol). Tables are stored as Hia[n*21 + coeff*3 + range] and
Hib[n*6 + k*3 + range].
"""
from __future__ import annotations

import json
import os

from .abi import Thermal, MAX_SPECIES

AVOGADRO = 6.02214076e26     # src/include/global_setup.h:49
BOLTZMANN = 1.380649e-23     # :51
RU = AVOGADRO * BOLTZMANN * 1.0E-3   # Ru, J/mol/K (:53-54)


def _tokens(path):
    with open(path, "r", encoding="latin-1") as f:
        return f.read().split()


def _find(tokens, name):
    key = "*" + name
    for n, t in enumerate(tokens):
        if t == "*END":
            break
        if t == key:
            return n + 1
    raise KeyError(f"species {name} not found")


def read_species_list(path, num_species):
    """First num_species names of a species_list.dat (ReadSpecies, thermal.cpp:14-20)."""
    return _tokens(path)[:num_species]


def read_tables(runtime_dir, species, thermo=1):
    """Return a dict {species, thermo, Wi_gmol, Hia, Hib} read from runtime.dat/ files."""
    ns = len(species)
    hia_nasa = [0.0] * (ns * 21)
    hib_nasa = [0.0] * (ns * 6)
    hia_janaf = [0.0] * (ns * 21)
    wi = [0.0] * ns
    tk = _tokens(os.path.join(runtime_dir, "thermal_dynamics.dat"))
    for n, name in enumerate(species):
        p = _find(tk, name)
        for rg in range(3):
            for m in range(7):
                hia_nasa[n * 21 + m * 3 + rg] = float(tk[p]); p += 1
            for m in range(2):
                hib_nasa[n * 6 + m * 3 + rg] = float(tk[p]); p += 1
        if thermo == 1:
            wi[n] = float(tk[p])
    tk = _tokens(os.path.join(runtime_dir, "thermal_dynamics_janaf.dat"))
    for n, name in enumerate(species):
        p = _find(tk, name)
        for rg in range(2):
            for m in range(7):
                hia_janaf[n * 21 + m * 3 + rg] = float(tk[p]); p += 1
        if thermo == 0:
            wi[n] = float(tk[p])
    return {
        "species": list(species), "thermo": int(thermo), "Wi_gmol": wi,
        "Hia": hia_nasa if thermo == 1 else hia_janaf,
        "Hib": hib_nasa if thermo == 1 else [0.0] * (ns * 6),
    }


def thermal_from_tables(tab) -> Thermal:
    """Build xfg_thermal: Wi *= 1e-3, _Wi = 1/Wi, Ri = Ru/Wi (thermal.cpp:169-173)."""
    ns = len(tab["species"])
    if ns > MAX_SPECIES:
        raise ValueError(f"{ns} species > {MAX_SPECIES}")
    t = Thermal()
    t.num_species = ns
    for n in range(ns):
        w = tab["Wi_gmol"][n] * 1e-3
        t.Wi[n] = w
        t._Wi[n] = 1.0 / w if w != 0.0 else float("inf")
        t.Ri[n] = RU / w if w != 0.0 else float("inf")
    for q, v in enumerate(tab["Hia"]):
        t.Hia[q] = v
    for q, v in enumerate(tab["Hib"]):
        t.Hib[q] = v
    return t


def load_thermal(species, thermo=1, runtime_dir=None, tables_json=None) -> Thermal:
    """Thermal for a species list, from runtime.dat files or from a tables JSON written by
    dump_tables()."""
    if tables_json is not None:
        with open(tables_json) as f:
            allt = json.load(f)
        tab = allt[f"{'+'.join(species)}:{thermo}"]
    else:
        tab = read_tables(runtime_dir, species, thermo)
    return thermal_from_tables(tab)


def dump_tables(runtime_dir, sets, path):
    """Write {"A+B+C:thermo": tables} for the given (species, thermo) sets."""
    out = {}
    for species, thermo in sets:
        out[f"{'+'.join(species)}:{thermo}"] = read_tables(runtime_dir, species, thermo)
    with open(path, "w") as f:
        json.dump(out, f, indent=1)


def transport_from_arrays(ns, visc, therm, dkj, chara, yil_limiter, dim_limiter):
    """xfg_transport from the fitted coefficients (ns x 4, ns x 4, ns*ns x 4), the species
    characteristics (ns x 9) and the two diffusion limiters."""
    import numpy as np

    from .abi import Transport
    t = Transport()
    t.num_species = int(ns)
    for name, a in (("visc", visc), ("therm", therm), ("dkj", dkj), ("species_chara", chara)):
        a = np.asarray(a, dtype=np.float64).reshape(-1)
        dst = getattr(t, name)
        for q, v in enumerate(a):
            dst[q] = float(v)
    t.yil_limiter, t.dim_limiter = float(yil_limiter), float(dim_limiter)
    return t


def load_transport(path):
    """xfg_transport from a file holding fitted transport data: an .npz with the arrays tr_visc
    (ns x 4), tr_therm (ns x 4), tr_dkj (ns*ns x 4), tr_chara (ns x 9) and tr_limits (Yil_limiter,
    Dim_limiter), as the golden fixtures of the viscous cases store the reference's fits."""
    import numpy as np
    z = np.load(path)
    ns = z["tr_chara"].size // 9
    return transport_from_arrays(ns, z["tr_visc"], z["tr_therm"], z["tr_dkj"], z["tr_chara"], *z["tr_limits"])
