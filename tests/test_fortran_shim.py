"""The Fortran side of the boundary (gom_release_gb300/fortran/gom_core_shim.f90) against the C
header and the ctypes binding: every bind(c) derived type has the header struct's fields in the
header's order with matching kinds, every bind(c) interface names a declared entry point with the
header's argument count, and the field ids and ABI version agree.  (No Fortran compiler exists
here, so the check is structural.)"""
import re
from pathlib import Path

from gom_release_gb300 import core

ROOT = Path(__file__).resolve().parent.parent
SHIM = ROOT / "gom_release_gb300" / "fortran" / "gom_core_shim.f90"
HEADER = ROOT / "include" / "gom_core.h"

STRUCTS = {"gom_dims": core.GomDims, "gom_params": core.GomParams, "gom_geom": core.GomGeom,
           "gom_forcing": core.GomForcing, "gom_status": core.GomStatus, "gom_series": core.GomSeries,
           "gom_boundary_series": core.GomBoundarySeries, "gom_mesh": core.GomMesh,
           "gom_mesh_geometry": core.GomMeshGeometry}


def _fortran_types():
    txt = SHIM.read_text()
    out = {}
    for m in re.finditer(r"type, bind\(c\) :: (\w+)\n(.*?)\n\s*end type", txt, re.S):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            kind, names = line.split("::")
            for n in re.findall(r"\w+(?:\(\d+\))?", names):
                dim = re.match(r"(\w+)(?:\((\d+)\))?", n)
                fields.append((kind.strip(), dim.group(1), int(dim.group(2) or 1)))
        out[m.group(1)] = fields
    return out


def _header_structs():
    txt = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \1;", txt, re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            first = re.match(r"(const\s+)?(\w+)\s+(.*)", decl, re.S)
            base = first.group(2)
            for part in first.group(3).split(","):
                part = part.strip()
                ptr = part.startswith("*")
                dim = re.match(r"(\w+)(?:\[(\d+)\])?", part.lstrip("*").strip())
                fields.append(("ptr" if ptr else base, dim.group(1), int(dim.group(2) or 1)))
        out[m.group(1)] = fields
    return out


def _kind_of(ctype):
    if hasattr(ctype, "_length_"):       # a fixed array: the element's kind
        return _kind_of(ctype._type_)
    if ctype is core.C.c_double:
        return "real(c_double)"
    if ctype is core.C.c_int32:
        return "integer(c_int32_t)"
    if ctype is core.GomSeries:
        return "type(gom_series)"
    return "type(c_ptr)"


def test_derived_types_match_header_and_ctypes():
    ft = _fortran_types()
    hs = _header_structs()
    cmap = {"double": "real(c_double)", "int32_t": "integer(c_int32_t)", "ptr": "type(c_ptr)",
            "gom_series": "type(gom_series)"}
    for name, cls in STRUCTS.items():
        assert name in ft, f"{name} missing from the Fortran binding"
        f_fields = ft[name]
        c_fields = [(_kind_of(t), n, getattr(t, "_length_", 1)) for n, t in cls._fields_]
        h_fields = [(cmap[k], n, c) for k, n, c in hs[name]]
        assert f_fields == c_fields, f"{name}: Fortran and ctypes differ"
        assert f_fields == h_fields, f"{name}: Fortran and header differ"


def test_interfaces_name_declared_entry_points_with_their_arity():
    txt = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    arity = {}
    for m in re.finditer(r"\b(gom_\w+)\s*\(([^;{]*?)\)\s*;", txt, re.S):
        args = m.group(2).strip()
        arity[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    shim = SHIM.read_text()
    found = re.findall(r"(?:function|subroutine) (\w+)\(([^)]*)\) bind\(c, name=\"(\w+)\"\)", shim)
    assert len(found) >= 20
    for fname, args, cname in found:
        assert fname == cname
        assert cname in arity, f"{cname} is not declared in the header"
        n = 0 if not args.strip() else len(args.split(","))
        assert n == arity[cname], f"{cname}: {n} arguments, header has {arity[cname]}"


def test_geometry_sites_match_header():
    shim = SHIM.read_text()
    sites = dict((n, int(v)) for n, v in re.findall(r"parameter :: GOM_GEO_(\w+) = (\d+)", shim))
    hdr = dict((n, int(v)) for n, v in re.findall(r"GOM_GEO_(\w+) = (\d+)", HEADER.read_text()))
    assert sites == hdr == core.GOM_GEO


def test_field_ids_and_abi_version():
    shim = SHIM.read_text()
    ids = dict((n.lower(), int(v)) for n, v in re.findall(r"parameter :: GOM_F_(\w+) = (\d+)", shim))
    assert ids == {n: i + 1 for i, n in enumerate(core.FIELDS)}
    v = int(re.search(r"GOM_ABI_VERSION = (\d+)", shim).group(1))
    assert v == core.ABI_VERSION == int(re.search(r"#define GOM_ABI_VERSION (\d+)", HEADER.read_text()).group(1))


def test_replacement_subroutines_keep_the_reference_names():
    shim = SHIM.read_text()
    for name in ("calculate_bottom_friction", "solve_nonlinear_advection", "solve_momentum_equation",
                 "solve_free_surface_equation", "solve_velocities", "update_vertical_layers_1",
                 "calculate_velocity_at_node", "solve_transport_equation_v19", "calculate_density_full",
                 "calculate_density_linear", "update_variables"):
        assert re.search(rf"^subroutine {name}\b", shim, re.M), name
