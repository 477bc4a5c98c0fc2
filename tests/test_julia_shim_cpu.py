"""The Julia shim (hypercloudcore.jl_gb300/julia/HCCGB300.jl), checked without Julia by reading it as text:

- every `const HCC_* = Int32(v)` equals the value of the same enum constant in include/hcc.h;
- its mirrors of hcc_config, hcc_mover, hcc_tuning and hcc_tune_report have the header's fields, in order, with the
  same element types and counts;
- every id mapping (`_limiter_id`, `_strategy_id`, `_flux_id`, `_bc_kind`, `_upwind_alg`, `_criterion`) returns a named
  header constant or raises, and the built-in tableau table covers every hcc_tableau value;
- each scheme method sets the fields the library reads (MUSCL: order, div_order, limiter, flux, moment correction);
- the stepper takes the tableau object and the grid's own boundary-condition map;
- where the reference sources are present, every reference name the shim calls exists there.
"""
import os
import re
from pathlib import Path

import pytest

from conftest import ROOT

JL = (ROOT / "hypercloudcore.jl_gb300" / "julia" / "HCCGB300.jl").read_text()
HDR = (ROOT / "include" / "hcc.h").read_text()
REF = Path(os.environ.get("HCC_REFERENCE_DIR", "/root/reference"))


def _header_enums():
    vals = {}
    for body in re.findall(r"typedef enum\s*\{(.*?)\}", HDR, re.S):
        for name, v in re.findall(r"(HCC_[A-Z0-9_]+)\s*=\s*(-?\d+)", body):
            vals[name] = int(v)
    return vals


def _julia_consts():
    out = {}
    for lhs, rhs in re.findall(r"(?m)^const\s+(HCC_[A-Z0-9_, ]+?)\s*=\s*(.+)$", JL):
        names = [n.strip() for n in lhs.split(",")]
        vals = re.findall(r"Int32\((-?\d+)\)", rhs)
        assert len(names) == len(vals), lhs
        out.update({n: int(v) for n, v in zip(names, vals)})
    return out


def test_constants_match_the_header():
    h, j = _header_enums(), _julia_consts()
    assert len(j) >= 35
    for name, v in j.items():
        assert name in h, name
        assert h[name] == v, (name, v, h[name])


C_SIZES = {"int32_t": ("Int32", 4), "double": ("Float64", 8)}
DIMS = {"HCC_MAX_DIM": 3, "HCC_MAX_TAGS": 16, "HCC_MAX_VARS": 16}


def _c_fields(struct):
    hdr = re.sub(r"/\*.*?\*/", "", HDR, flags=re.S)          # comments may hold braces
    m = re.search(r"typedef struct(?:\s+\w+)?\s*\{([^{}]*)\}\s*" + struct + r";", hdr)
    assert m, struct
    out = []
    for typ, names in re.findall(r"(int32_t|double|hcc_tuning)\s+([^;]+);", m.group(1)):
        for nm in names.split(","):
            nm = nm.strip()
            count = 1
            for dim in re.findall(r"\[(\w+)\]", nm):
                count *= DIMS.get(dim, int(dim) if dim.isdigit() else 0)
            out.append((nm.split("[")[0], typ, count))
    return out


def _jl_fields(struct):
    m = re.search(r"(?:mutable\s+)?struct\s+" + struct + r"\b(.*?)\n\s*(?:Hcc\w+\(\)\s*=.*\n)?end\b", JL, re.S)
    assert m, struct
    out = []
    for nm, typ in re.findall(r"(\w+)::([\w{}, ]+?)(?=[;\n]|\s+#)", m.group(1) + "\n"):
        t = re.match(r"NTuple\{(\d+),\s*(\w+)\}", typ)
        out.append((nm, t.group(2), int(t.group(1))) if t else (nm, typ.strip(), 1))
    return out


@pytest.mark.parametrize("c_name,jl_name", [("hcc_config", "HccConfig"), ("hcc_mover", "HccMover"),
                                            ("hcc_tuning", "HccTuning"), ("hcc_tune_report", "HccTuneReport")])
def test_struct_mirrors_match_the_header(c_name, jl_name):
    cf, jf = _c_fields(c_name), _jl_fields(jl_name)
    assert [f[0] for f in cf] == [f[0] for f in jf], (c_name, [f[0] for f in cf], [f[0] for f in jf])
    for (n, ct, cc), (_, jt, jc) in zip(cf, jf):
        if ct == "hcc_tuning":
            assert jt == "HccTuning", n
            continue
        assert C_SIZES[ct][0] == jt and cc == jc, (n, ct, cc, jt, jc)


def test_id_mappings_return_header_constants():
    h = _header_enums()
    for fn in ("_limiter_id", "_strategy_id", "_flux_id", "_bc_kind", "_upwind_alg"):
        methods = re.findall(r"(?m)^" + fn + r"\((.*?)\)\s*=\s*(.+)$", JL)
        assert methods, fn
        for arg, rhs in methods:
            rhs = rhs.strip()
            assert rhs.startswith("error(") or rhs in h, (fn, arg, rhs)
    crit = re.findall(r"(?m)^_criterion\(.*?\)\s*=\s*\((HCC_[A-Z0-9_]+),", JL)
    assert sorted(crit) == sorted(["HCC_MOOD_U1", "HCC_MOOD_U2", "HCC_MOOD_PAD", "HCC_MOOD_ONLY", "HCC_MOOD_NONE"])
    assert re.search(r"_limiter_id\(::VenkatakrishnanLimiter\{:hard\}\)\s*=\s*HCC_LIMITER_VK_HARD", JL)
    assert re.search(r"_strategy_id\(::EPD1\)\s*=\s*HCC_EPD1", JL)
    assert re.search(r"_bc_kind\(::OutflowBC\)\s*=\s*HCC_BC_OUTFLOW", JL)
    assert re.search(r"_bc_kind\(::FixedDirichlet\)\s*=\s*HCC_BC_DIRICHLET", JL)


def test_builtin_tableau_table_covers_every_tableau():
    h = _header_enums()
    tab = re.search(r"_BUILTIN_TABLEAUS\s*=\s*\((.*?)\)\)\n", JL, re.S).group(1)
    pairs = re.findall(r"HyperCloudCore\.(\w+),\s*(HCC_TAB_\w+)", tab)
    assert sorted(v for _, v in pairs) == sorted(k for k in h if k.startswith("HCC_TAB_"))
    for builder, const in pairs:              # RK3_SSP_Tableau <-> HCC_TAB_RK3_SSP
        assert builder.replace("_Tableau", "").upper() == const.replace("HCC_TAB_", ""), (builder, const)
    assert re.search(r"function _tableau_id\(bt::HyperCloudCore\.IMEXButcherTableau", JL)


def test_scheme_methods_set_the_fields_the_library_reads():
    bodies = dict(re.findall(r"function _scheme!\(cfg, [^:]*::(\w+)\{.*?\n(.*?)\nend", JL, re.S))
    assert set(bodies) >= {"MUSCL", "WENO", "CentralDivergence", "UpwindDivergence"}
    for key in ("cfg.scheme", "cfg.muscl_order", "cfg.div_order = DIV_ORDER", "cfg.limiter", "cfg.flux",
                "cfg.moment_correction"):
        assert key in bodies["MUSCL"], key
    for name in ("WENO", "CentralDivergence", "UpwindDivergence"):
        assert "DIV_ORDER" in bodies[name] and "cfg.muscl_order" in bodies[name], name
    assert "cfg.upwind_algorithm" in bodies["UpwindDivergence"]


def test_stepper_takes_the_tableau_object_and_the_grid_bc_map():
    ctor = re.search(r"function GB300RKTimeStepper\((.*?)\nend", JL, re.S).group(1)
    assert "cfg.tableau = _tableau_id(tableau)" in ctor
    assert "pg.geometry.bc_map" in ctor and "_bc_by_tag(" in ctor
    assert "_scheme!(cfg, interp)" in ctor
    builder = re.search(r"function build_gb300_timestepper\((.*?)\nend", JL, re.S).group(1)
    assert "context[:Tableau]" in builder and "_tableau_id(context" not in builder


def test_reference_names_exist():
    if not (REF / "src").is_dir():
        pytest.skip("reference sources not present")
    src = "\n".join(p.read_text(errors="replace") for p in (REF / "src").rglob("*.jl"))
    for name in ("FixedDirichlet", "OutflowBC", "IMEXButcherTableau", "RK1_Euler_Tableau", "RK2_SSP_Tableau",
                 "RK2_Ralston_Tableau", "RK3_SSP_Tableau", "RK4_Classical_Tableau", "RK4_SSP_Tableau",
                 "IMEX_Euler_Tableau", "IMEX_ARS233_Tableau", "IMEX_ARS222_Tableau", "IMEX_PRSSP3_Tableau",
                 "IMEX_SSP2332_Tableau", "struct MUSCL", "struct WENO", "struct CentralDivergence",
                 "struct UpwindDivergence", "TiwariAlgorithm", "PraveenAlgorithm", "ClassicAlgorithm",
                 "VenkatakrishnanLimiter", "BarthJespersenLimiter", "AlignedRusanovFlux", "StrictEPD0", "MOODu2",
                 "streamed::", "moment_correction"):
        assert name in src, name
    # type-parameter positions the shim's methods rely on
    assert re.search(r"struct MUSCL\{D, M, T, B_LEN, MAX_ORDER, DIV_ORDER", src)
    assert re.search(r"struct WENO\{D, M, T, MAX_ORDER, DIV_ORDER", src)
    assert re.search(r"struct CentralDivergence\{D, M, T, MAX_ORDER, DIV_ORDER", src)
    assert re.search(r"struct UpwindDivergence\{D, M, T, MAX_ORDER, DIV_ORDER, B_LEN, INTERPS, Algorithm", src)
