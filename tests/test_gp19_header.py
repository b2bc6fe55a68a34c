"""GP19 tables in the reference's header format (GP19Table.hpp, included by
kernel_brem_GP19.hpp): the host parser and the library loader."""

import numpy as np
import pytest

import bns_nurates_gb300 as bn
from bns_nurates_gb300 import gp19_synthetic


def write_header(path, tab, with_logs=True):
    """A header laid out like a generated GP19Table.hpp: constexpr dims and
    brace-initialised arrays, with comments, float suffixes and a nested
    initialiser for the data."""
    d = tab["dims"]

    def arr(name, size, vals, nested=False):
        body = ",\n  ".join(", ".join(f"{v:.17g}" for v in vals[i:i + 6])
                            for i in range(0, len(vals), 6))
        if nested:
            w = d[3]
            body = ",\n".join("{" + ", ".join(f"{v:.17g}" for v in vals[i:i + w]) + "}"
                              for i in range(0, len(vals), w))
        return f"constexpr BS_REAL {name}[{size}] = {{\n  {body}\n}};\n"

    out = ["// GP19 response table (test copy)\n", "#pragma once\n",
           f"constexpr int GP19_nb_dims = {d[0]};  // nb\n",
           f"constexpr int GP19_Ye_dims = {d[1]};\n",
           f"constexpr int GP19_T_dims = {d[2]}; /* T */\n",
           f"constexpr int GP19_w_dims = {d[3]};\n",
           arr("GP19_nb_axis", "GP19_nb_dims", tab["nb"]),
           arr("GP19_Ye_axis", "GP19_Ye_dims", tab["ye"]),
           arr("GP19_T_axis", "GP19_T_dims", tab["t"]),
           arr("GP19_w_axis", "GP19_w_dims", tab["w"])]
    if with_logs:
        out += [arr("GP19_lognb_axis", "GP19_nb_dims", np.log(tab["nb"])),
                arr("GP19_logw_axis", "GP19_w_dims", np.log(tab["w"]))]
    out.append(arr("GP19_data", "GP19_nb_dims * GP19_Ye_dims * GP19_T_dims * GP19_w_dims",
                   tab["data"], nested=True))
    open(path, "w").write("".join(out))


def test_header_parser_round_trip(tmp_path):
    tab = gp19_synthetic.table()
    p = tmp_path / "GP19Table.hpp"
    write_header(p, tab)
    got = bn.gp19_table_from_header(p)
    assert tuple(got["dims"]) == tuple(tab["dims"])
    for k in ("nb", "ye", "t", "w", "data"):
        assert np.array_equal(got[k], np.asarray(tab[k], dtype=np.float64)), k
    assert np.array_equal(got["lognb"], np.log(tab["nb"]))
    write_header(p, tab, with_logs=False)
    got = bn.gp19_table_from_header(p)
    assert got["lognb"] is None and got["logw"] is None


def test_header_parser_rejects_short_arrays(tmp_path):
    tab = dict(gp19_synthetic.table())
    tab["data"] = np.asarray(tab["data"])[:-1]
    p = tmp_path / "bad.hpp"
    write_header(p, tab)
    with pytest.raises(ValueError):
        bn.gp19_table_from_header(p)


@pytest.mark.gpu
def test_library_loader_matches_set_table(cuda, tmp_path):
    tab = gp19_synthetic.table()
    p = tmp_path / "GP19Table.hpp"
    write_header(p, tab)
    eos, m1 = bn.synthetic_points(77, 2000)
    e, m = cuda.from_numpy(eos).cuda(), cuda.from_numpy(m1).cuda()
    pars = bn.opacity_params(True, False, True, True, True, brem_implementation=2)
    q = bn.gauss_legendre(10)
    bn.set_gp19_table(tab)
    a = bn.m1_opacities(e, m, bn.opacity_flags(), pars, q).cpu().numpy()
    bn.load_gp19_header(p)
    b = bn.m1_opacities(e, m, bn.opacity_flags(), pars, q).cpu().numpy()
    assert np.array_equal(a, b)
    with pytest.raises(bn.BnsnError):
        bn.load_gp19_header(tmp_path / "missing.hpp")
    bn.set_gp19_table(__import__("oracle")._synthetic_gp19())
