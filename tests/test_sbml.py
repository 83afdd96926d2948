"""SBML import (lassie_gb300/sbml.py): mass-action models in the level-1
formula form LASSIE's own example model uses and in level-2/3 MathML, the
converter to the input-folder format, and the rejections."""
import os
import subprocess
import sys

import numpy as np
import pytest

from lassie_gb300 import sbml
from lassie_gb300.model import load_folder

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

L1 = """<?xml version="1.0" encoding="UTF-8"?>
<sbml xmlns="http://www.sbml.org/sbml/level1" level="1" version="2">
 <model name="m">
  <listOfCompartments><compartment name="c"/></listOfCompartments>
  <listOfSpecies>
   <species name="A" compartment="c" initialAmount="0.5"/>
   <species name="B" compartment="c" initialAmount="1.5"/>
   <species name="C" compartment="c" initialAmount="0"/>
  </listOfSpecies>
  <listOfReactions>
   <reaction name="R0" reversible="false">
    <listOfReactants>
     <speciesReference species="A" stoichiometry="1"/>
     <speciesReference species="B" stoichiometry="1"/>
    </listOfReactants>
    <listOfProducts><speciesReference species="C" stoichiometry="2"/></listOfProducts>
    <kineticLaw formula="K0* A* B">
     <listOfParameters><parameter name="K0" value="2.5E-1"/></listOfParameters>
    </kineticLaw>
   </reaction>
   <reaction name="R1" reversible="false">
    <listOfReactants><speciesReference species="C" stoichiometry="2"/></listOfReactants>
    <kineticLaw formula="K1*C^2">
     <listOfParameters><parameter name="K1" value="3"/></listOfParameters>
    </kineticLaw>
   </reaction>
  </listOfReactions>
 </model>
</sbml>"""

L3 = """<?xml version="1.0" encoding="UTF-8"?>
<sbml xmlns="http://www.sbml.org/sbml/level3/version1/core" level="3" version="1">
 <model id="m">
  <listOfCompartments><compartment id="cell" size="1" constant="true"/></listOfCompartments>
  <listOfSpecies>
   <species id="X" compartment="cell" initialConcentration="2"/>
   <species id="Y" compartment="cell" initialConcentration="0"/>
  </listOfSpecies>
  <listOfParameters><parameter id="kf" value="0.7" constant="true"/></listOfParameters>
  <listOfReactions>
   <reaction id="r" reversible="false">
    <listOfReactants><speciesReference species="X" stoichiometry="1"/></listOfReactants>
    <listOfProducts><speciesReference species="Y" stoichiometry="1"/></listOfProducts>
    <kineticLaw>
     <math xmlns="http://www.w3.org/1998/Math/MathML">
      <apply><times/><ci>cell</ci><ci>kf</ci><ci>X</ci></apply>
     </math>
    </kineticLaw>
   </reaction>
   <reaction id="src" reversible="false">
    <listOfProducts><speciesReference species="X" stoichiometry="1"/></listOfProducts>
    <kineticLaw><math xmlns="http://www.w3.org/1998/Math/MathML"><cn>0.25</cn></math></kineticLaw>
   </reaction>
  </listOfReactions>
 </model>
</sbml>"""


@pytest.mark.parametrize("strict", [False, True])
def test_level1_formula_model(strict):
    m = sbml.read_sbml(L1, t=np.linspace(0, 1, 5), strict=strict)
    assert m.left.tolist() == [[1, 1, 0], [0, 0, 2]]
    assert m.right.tolist() == [[0, 0, 2], [0, 0, 0]]
    assert np.allclose(m.k, [0.25, 3.0])
    assert m.x0.tolist() == [0.5, 1.5, 0.0]


@pytest.mark.parametrize("strict", [False, True])
def test_level3_mathml_model(strict):
    m = sbml.read_sbml(L3, strict=strict)
    assert m.left.tolist() == [[1, 0], [0, 0]]
    assert m.right.tolist() == [[0, 1], [1, 0]]
    assert np.allclose(m.k, [0.7, 0.25])
    assert m.x0.tolist() == [2.0, 0.0]


def test_rate_constant_as_lassies_converter_takes_it():
    """Default: k is the law's one parameter whatever the formula, as
    LASSIE's own converter does (a stochastic-style 2C law included)."""
    law = L1.replace('formula="K1*C^2"', 'formula="K1* (1/2) * C* (C-1)"')
    m = sbml.read_sbml(law)
    assert np.allclose(m.k, [0.25, 3.0])
    with pytest.raises(sbml.SbmlError):
        sbml.read_sbml(law, strict=True)


@pytest.mark.parametrize("bad,what,strict", [
    (L1.replace('formula="K0* A* B"', 'formula="K0* A"'), "not mass action", True),
    (L1.replace('formula="K1*C^2"', 'formula="K1*C/(1+C)"'), "mass-action product", True),
    (L1.replace('name="R1" reversible="false"', 'name="R1" reversible="true"'), "reversible", False),
    (L1.replace('formula="K0* A* B"', 'formula="K9* A* B"'), "unknown symbol", True),
    (L1.replace('formula="K0* A* B"', 'formula="K0* K2* A* B"').replace(
        '<parameter name="K0" value="2.5E-1"/>',
        '<parameter name="K0" value="2.5E-1"/><parameter name="K2" value="2"/>'),
     "names 2 parameters", False),
])
def test_rejections_name_the_reaction(bad, what, strict):
    with pytest.raises(sbml.SbmlError) as e:
        sbml.read_sbml(bad, strict=strict)
    assert what in str(e.value) and "reaction R" in str(e.value)


def test_converter_writes_an_input_folder(tmp_path):
    src = tmp_path / "m.sbml"
    src.write_text(L1)
    out = tmp_path / "folder"
    r = subprocess.run([sys.executable, "-m", "lassie_gb300.sbml", str(src), str(out),
                        "--t-end", "2", "--samples", "3"], cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    m = load_folder(str(out))
    assert m.left.tolist() == [[1, 1, 0], [0, 0, 2]]
    assert np.allclose(m.k, [0.25, 3.0])
    assert np.allclose(m.t, [0, 1, 2])


@pytest.mark.parametrize("strict", [False, True])
def test_write_read_round_trip(strict):
    from lassie_gb300 import synth
    m = synth.make_c1()
    back = sbml.read_sbml(sbml.write_sbml(m), t=m.t, strict=strict)
    assert np.array_equal(back.left, m.left) and np.array_equal(back.right, m.right)
    assert np.array_equal(back.k, m.k) and np.array_equal(back.x0, m.x0)


REV_L2 = """<?xml version="1.0" encoding="UTF-8"?>
<sbml xmlns="http://www.sbml.org/sbml/level2/version4" level="2" version="4">
 <model id="rev">
  <listOfCompartments><compartment id="c" size="1"/></listOfCompartments>
  <listOfSpecies>
   <species id="A" compartment="c" initialConcentration="1.0"/>
   <species id="B" compartment="c" initialConcentration="0.5"/>
   <species id="C" compartment="c" initialConcentration="0.0"/>
   <species id="E" compartment="c" initialConcentration="2.0" constant="true"/>
  </listOfSpecies>
  <listOfParameters>
   <parameter id="kf" value="2.0"/><parameter id="kr" value="0.25"/>
   <parameter id="kd" value="0.1"/>
  </listOfParameters>
  <listOfReactions>
   <reaction id="bind">
    <listOfReactants>
     <speciesReference species="A"/><speciesReference species="B"/>
    </listOfReactants>
    <listOfProducts><speciesReference species="C"/></listOfProducts>
    <kineticLaw><math xmlns="http://www.w3.org/1998/Math/MathML">
     <apply><minus/>
      <apply><times/><ci>kf</ci><ci>A</ci><ci>B</ci></apply>
      <apply><times/><ci>kr</ci><ci>C</ci></apply>
     </apply></math></kineticLaw>
   </reaction>
   <reaction id="decay" reversible="false">
    <listOfReactants><speciesReference species="C"/></listOfReactants>
    <listOfProducts><speciesReference species="E"/></listOfProducts>
    <kineticLaw><math xmlns="http://www.w3.org/1998/Math/MathML">
     <apply><times/><ci>kd</ci><ci>C</ci></apply></math></kineticLaw>
   </reaction>
  </listOfReactions>
 </model>
</sbml>
"""


@pytest.mark.parametrize("strict", [False, True])
def test_reversible_reaction_is_split(strict):
    """SBML2BSW.py:191-197,245-290: a reversible reaction becomes the forward
    reaction followed by the reverse one (reactants and products swapped),
    with the first and second rate constants of its law."""
    m = sbml.read_sbml(REV_L2, strict=strict)
    assert m.left.tolist() == [[1, 1, 0, 0], [0, 0, 1, 0], [0, 0, 1, 0]]
    assert m.right.tolist() == [[0, 0, 1, 0], [1, 1, 0, 0], [0, 0, 0, 1]]
    assert np.allclose(m.k, [2.0, 0.25, 0.1])


def test_reversible_declared_in_level1_formula():
    law = L1.replace('name="R0" reversible="false"', 'name="R0" reversible="true"').replace(
        'formula="K0* A* B"', 'formula="K0* A* B - K2* C* C"').replace(
        '<parameter name="K0" value="2.5E-1"/>',
        '<parameter name="K0" value="2.5E-1"/><parameter name="K2" value="4"/>')
    for strict in (False, True):
        m = sbml.read_sbml(law, strict=strict)
        assert m.left.tolist() == [[1, 1, 0], [0, 0, 2], [0, 0, 2]]
        assert m.right.tolist() == [[0, 0, 2], [1, 1, 0], [0, 0, 0]]
        assert np.allclose(m.k, [0.25, 4.0, 3.0])


def test_constant_species_are_fed():
    """SBML2BSW.py:302-305: constant species are written to M_feed (value 1
    as the converter writes it, or the initial amount on request)."""
    m = sbml.read_sbml(REV_L2)
    assert m.feed.tolist() == [0.0, 0.0, 0.0, 1.0]
    m2 = sbml.read_sbml(REV_L2, feed="initial")
    assert m2.feed.tolist() == [0.0, 0.0, 0.0, 2.0]
    assert sbml.read_sbml(L1).feed is None


def test_split_model_conserves_moieties_in_the_oracle():
    """A + B <-> C (split) then C -> E with E fed: A + C + (C consumed) --
    here A - B stays constant, and E stays at its feed value."""
    from oracle import oracle as O
    m = sbml.read_sbml(REV_L2, t=np.linspace(0.0, 2.0, 5), feed="initial")
    out, _, rc = O.solve(m)
    assert rc == 0
    a, b, c, e = out.T
    assert np.allclose(a - b, a[0] - b[0], rtol=0, atol=1e-9)
    assert np.all(e[1:] == 2.0)
    assert c[-1] > 0


def test_converter_writes_m_feed(tmp_path):
    src = tmp_path / "rev.sbml"
    src.write_text(REV_L2)
    out = tmp_path / "folder"
    r = subprocess.run([sys.executable, "-m", "lassie_gb300.sbml", str(src), str(out),
                        "--feed", "initial"], cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    m = load_folder(str(out))
    assert m.n_reactions == 3
    assert m.feed.tolist() == [0.0, 0.0, 0.0, 2.0]
