"""Host-side logic through the C ABI (no GPU needed): exported symbols, model
tables derived like the reference's load toolchain, StochKit reading and
writing, the seeded generator, and error reporting."""
import re
from pathlib import Path

import numpy as np
import pytest

from tau_leaping_gb300 import Model, TLError, _ffi

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "tl.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tl_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _ffi.lib()
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"libtl.so does not export {n}"
    assert set(names) == set(_ffi.SIGNATURES), "binding table out of sync with include/tl.h"
    assert lib.tl_abi_version() == 2
    for s in range(13):
        assert lib.tl_status_str(s)


def test_integration_binding_compiles_and_links(tmp_path):
    """The C++ `Model` class a maintainer of the reference adds
    (tau_leaping_gb300/host/gpu_model.h) builds against include/tl.h and
    links against libtl.so."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    (tmp_path / "main.cpp").write_text(
        '#include "gpu_model.h"\n'
        "int main(int argc, char** argv) {\n"
        "    if (argc < 2) return 0;\n"
        "    std::vector<std::string> names;\n"
        "    Model* m = Model::ReadXML(argv[1], names);\n"
        "    std::vector<char> track(m->ReactantsCount(), 1);\n"
        "    std::vector<double> mean, sd, t;\n"
        "    m->PerformCalcAll(0.1f, 0.03f, track, 100, 2, 0x7fffffff, 1, mean, sd, t);\n"
        "    delete m;\n"
        "}\n")
    lib = ROOT / "tau_leaping_gb300"
    r = subprocess.run([gxx, "-std=c++17", "-I", str(ROOT / "include"), "-I", str(lib / "host"),
                        str(tmp_path / "main.cpp"), "-L", str(lib),
                        "-ltl", f"-Wl,-rpath,{lib}", "-o", str(tmp_path / "a.out")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(tmp_path / "a.out")]).returncode == 0  # no model given: exits before any GPU call


def dimer_arrays(s1=100000):
    # channel-major entries exactly as ReadXMLToMatrixStruct would list them
    col_ptr = [0, 1, 3, 5, 7]
    row = [0, 0, 1, 0, 1, 1, 2]
    v = [-1, -2, 1, 2, -1, -1, 1]
    return [s1, 0, 0], [1.0, 0.002, 0.5, 0.04], col_ptr, row, v


def test_dimer_tables_match_reference_layout():
    m = Model.from_arrays(*dimer_arrays())
    t = m.tables()
    assert t["order"].tolist() == [1, 3, 1, 1]
    assert t["s0"].tolist() == [0, 0, 1, 1]
    # species-row CSR, reference packing (col<<3)|((v+2)&7)
    assert t["csr_row_ptr"].tolist() == [0, 3, 6, 7]
    assert t["csr_valcol"].tolist() == [1, 8, 20, 11, 17, 25, 27]
    assert (m.n_species, m.n_channels, m.nnz_raw, m.nnz_net) == (3, 4, 7, 7)
    assert m.pop_bits == 32


def test_generator_matches_xml_builder(tmp_path):
    g = Model.generate("dimer")
    d = g.desc()
    x0, rate, cp, row, v = dimer_arrays()
    assert d["x0"].tolist() == x0
    assert np.allclose(d["rate"], rate)
    assert d["col_ptr"].tolist() == cp
    assert d["row_ind"].tolist() == row
    assert d["stoich"].tolist() == v
    p = tmp_path / "dimer.xml"
    g.write_stochkit(p)
    m2 = Model.from_stochkit(p)
    d2 = m2.desc()
    for k in d:
        assert np.array_equal(d[k], d2[k]), k
    assert m2.species_names() == ["S1", "S2", "S3"]


XML_QUIRKS = """<?xml version="1.0"?>
<!-- quirks the reference's reader accepts -->
<Model>
  <NumberOfReactions>3</NumberOfReactions>
  <NumberOfSpecies>3</NumberOfSpecies>
  <ParametersList>
    <Parameter><Id>k1</Id><Expression>0.5</Expression></Parameter>
    <Parameter><Id>k2</Id><Expression> 2e-3 </Expression></Parameter>
  </ParametersList>
  <ReactionsList>
    <Reaction><Id>R1</Id><Rate>k1</Rate>
      <Reactants><SpeciesReference id="B" stoichiometry="1"/></Reactants>
    </Reaction>
    <Reaction><Id>R2</Id><Rate>k2</Rate>
      <Reactants><SpeciesReference id="A" stoichiometry="1"/><SpeciesReference id="C" stoichiometry="1"/></Reactants>
      <Products><SpeciesReference id="A" stoichiometry="2"/></Products>
    </Reaction>
    <Reaction><Id>R3</Id><Rate>0.25</Rate>
      <Reactants></Reactants>
      <Products><SpeciesReference id="C" stoichiometry="1"/></Products>
    </Reaction>
  </ReactionsList>
  <SpeciesList>
    <Species><Id>C</Id><InitialPopulation>7</InitialPopulation></Species>
    <Species><Id>A</Id><InitialPopulation>100</InitialPopulation></Species>
    <Species><Id>B</Id><InitialPopulation>3000000000</InitialPopulation></Species>
  </SpeciesList>
</Model>
"""


def test_stochkit_quirks(tmp_path):
    p = tmp_path / "q.xml"
    p.write_text(XML_QUIRKS)
    m = Model.from_stochkit(p)
    assert m.species_names() == ["C", "A", "B"]          # index = SpeciesList order
    assert m.pop_bits == 64                              # 3e9 needs 64-bit populations
    d = m.desc()
    assert d["x0"].tolist() == [7, 100, 3000000000]
    assert np.allclose(d["rate"], [0.5, 2e-3, 0.25])     # numeric <Rate> accepted
    # R2: rows sorted (C=0, A=1, A=1): C reactant, A reactant then A product
    assert d["col_ptr"].tolist() == [0, 1, 4, 5]
    assert d["row_ind"].tolist() == [2, 0, 1, 1, 0]
    assert d["stoich"].tolist() == [-1, -1, -1, 2, 1]
    t = m.tables()
    assert t["order"].tolist() == [1, 2, 0]
    assert (m.nnz_raw, m.nnz_net) == (5, 4)              # A: -1 + 2 merges to +1


@pytest.mark.parametrize("bad,status", [
    ("<Model><NumberOfReactions>1</NumberOfReactions></Model>", 11),
    ("<Model><NumberOfReactions>2", 11),
])
def test_stochkit_errors(tmp_path, bad, status):
    p = tmp_path / "bad.xml"
    p.write_text(bad)
    with pytest.raises(TLError) as e:
        Model.from_stochkit(p)
    assert e.value.status == status
    with pytest.raises(TLError) as e:
        Model.from_stochkit(tmp_path / "missing.xml")
    assert e.value.status == 10


def test_invalid_models_rejected():
    x0, rate, cp, row, v = dimer_arrays()
    with pytest.raises(TLError) as e:
        Model.from_arrays([-1, 0, 0], rate, cp, row, v)
    assert e.value.status == 2
    with pytest.raises(TLError) as e:
        Model.from_arrays(x0, [1.0, -0.1, 0.5, 0.04], cp, row, v)
    assert e.value.status == 12
    with pytest.raises(TLError) as e:   # 3S -> : third-order, unsupported
        Model.from_arrays([10], [1.0], [0, 1], [0], [-3])
    assert e.value.status == 3
    with pytest.raises(TLError) as e:   # species index out of range
        Model.from_arrays(x0, rate, cp, [0, 0, 1, 0, 1, 1, 3], v)
    assert e.value.status == 2
    with pytest.raises(TLError) as e:   # int32 requested but x0 needs int64
        Model.from_arrays([2**33, 0, 0], rate, cp, row, v, pop_bits=32)
    assert e.value.status == 4


def test_colloid_generator_structure():
    m = Model.generate("colloid")
    assert (m.n_species, m.n_channels, m.nnz_raw, m.nnz_net) == (250, 31250, 93500, 93500)
    assert m.pop_bits == 64
    t = m.tables()
    rp = t["csr_row_ptr"]
    assert int(np.diff(rp).max()) == 498 or int(np.diff(rp).max()) > 300
    d = m.desc()
    assert d["x0"].min() >= 1000 and d["x0"].max() <= 2000
    assert set(np.round(d["rate"], 6)) == {1e-4, 0.1}


def test_chain_and_toy_generators_are_seeded():
    c = Model.generate("chain")
    assert (c.n_species, c.n_channels, c.nnz_net) == (1024, 1024, 2048)
    a = Model.generate("toy").desc()
    b = Model.generate("toy").desc()
    for k in a:
        assert np.array_equal(a[k], b[k])
    c2 = Model.generate("toy", seed=8).desc()
    assert not np.array_equal(a["x0"], c2["x0"])
    t = Model.generate("toy")
    assert (t.n_species, t.n_channels) == (128, 256)
    o = t.tables()["order"]
    assert set(o.tolist()) <= {1, 2, 3}
    assert a["x0"].min() >= 0 and a["x0"].max() <= 10000
    assert a["rate"].min() >= 1e-3 and a["rate"].max() <= 1.0
    # every species is used by some channel
    assert len(set(a["row_ind"].tolist())) == 128
