"""Block geometry as the reference's Setup::init computes it (src/read_ini/src/iniset.cpp:290-369)."""
from __future__ import annotations

from .abi import Block, Scheme, Thermal, PERIODIC, OUTFLOW, LLF


def make_block(resolution, domain_size, boundarys, cfl=0.5, bwidth=4, domain_min=(0.0, 0.0, 0.0)) -> Block:
    """Mirror of Setup::init for one rank (mx = my = mz = 1).

    resolution: (X_inner, Y_inner, Z_inner) with 0 for an absent dimension (JSON "Resolution").
    domain_size: (length, width, height) (JSON "DOMAIN_Size").
    boundarys: six BConditions ids XMIN..ZMAX (JSON "Boundarys").
    bwidth: ghost layers, the JSON default Bwidth = 4 (src/read_ini/settings/read_json.cpp:115).
    """
    b = Block()
    dims = [int(r > 0) for r in resolution]
    inner = [int(r) if d else 1 for r, d in zip(resolution, dims)]
    bw = [bwidth if d else 0 for d in dims]
    length = [float(s) if d else 1.0 for s, d in zip(domain_size, dims)]
    b.DimX, b.DimY, b.DimZ = dims
    b.X_inner, b.Y_inner, b.Z_inner = inner
    b.Bwidth_X, b.Bwidth_Y, b.Bwidth_Z = bw
    b.Xmax, b.Ymax, b.Zmax = [n + 2 * w if d else 1 for n, w, d in zip(inner, bw, dims)]
    sp = [length[a] / float(inner[a]) if dims[a] else 1.0 for a in range(3)]
    b.dx, b.dy, b.dz = sp
    b._dx, b._dy, b._dz = [1.0 / s for s in sp]
    b.CFLnumber = float(cfl)
    for n in range(6):
        b.Boundarys[n] = int(boundarys[n])
    return b


def make_scheme(cop=False, num_species=1, scheme_order=5, artificial_type=LLF, thermo=1,
                ghost_species=False, ncop_gamma=1.4, precision=0, positivity=False) -> Scheme:
    s = Scheme()
    s.cop = int(bool(cop))
    s.num_species = int(num_species) if cop else 1
    s.scheme_order = int(scheme_order)
    s.artificial_type = int(artificial_type)
    s.thermo = int(thermo)
    s.ghost_species = int(bool(ghost_species))
    s.ncop_gamma = float(ncop_gamma)
    s.precision = int(precision)
    s.positivity = int(bool(positivity))
    return s


def empty_thermal(num_species=1) -> Thermal:
    t = Thermal()
    t.num_species = num_species
    return t


def block_cells(b: Block) -> int:
    return b.Xmax * b.Ymax * b.Zmax


__all__ = ["make_block", "make_scheme", "empty_thermal", "block_cells", "PERIODIC", "OUTFLOW"]
