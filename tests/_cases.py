"""Shared loaders that rebuild the golden cases' inputs from their seeds."""
import numpy as np

from slakonet_gb300 import synthetic as syn

CASES = ["si_cfg0", "si_klines", "rand_f4", "rand_a", "rand_b", "rand_c"]


def tables_checksum(tables):
    acc = []
    for pk in sorted(tables["pairs"]):
        for kind in ("H", "S"):
            for key in sorted(tables["pairs"][pk][kind]):
                t = tables["pairs"][pk][kind][key]
                acc.append([np.abs(t).sum(), t[:, 100].sum(), t[:, -1].sum()])
    for z in sorted(tables["elements"]):
        acc.append([np.sum(tables["elements"][z]["on_sites"]), np.sum(tables["elements"][z]["occupations"]), 0.0])
    return np.array(acc)


def load_case(g):
    """(structure, tables, shell_dict) for a golden case; checks the table checksum."""
    st = {"numbers": g["numbers"], "positions": g["positions"], "cell": g["cell"]}
    if "shells" in g.files:
        sd = {14: [int(x) for x in g["shells"]]}
        tables = syn.make_tables([14], sd, seed=int(g["seed"]))
    else:
        sd = syn.default_shell_dict()
        tables = syn.make_tables(st["numbers"], sd, seed=int(g["table_seed"]))
        sd = {int(z): sd[int(z)] for z in st["numbers"]}
    # numpy's exp differs by an ulp between x86 and aarch64 builds, so the regenerated
    # tables match the fixture's to rounding, not bit for bit
    np.testing.assert_allclose(tables_checksum(tables), g["tables_checksum"], rtol=1e-12, atol=1e-300)
    return st, tables, sd
