"""SBML import for mass-action networks (python3, standard library only).

LASSIE converts SBML with libsbml in its GUI (``gui/SBML2BSW.py:163-330``)
into its input-folder format.  This module reads the same kind of model
without libsbml: SBML levels 1-3, species by ``id`` (``name`` in level 1),
``initialAmount`` or ``initialConcentration``, integer stoichiometries.  The
rate constant follows LASSIE's converter (``gui/SBML2BSW.py:176-230``): the
one parameter (local or global) that the kinetic law names, whatever the
rest of the formula -- so a stochastic-style law ``K*(1/2)*X*(X-1)`` gives
k = K with X of stoichiometry 2 in the reactants.  With ``strict=True`` the
law must instead be a mass-action product (constants times each reactant to
the power of its stoichiometry) and k is the product of its constants.

Reversible reactions are split in two, as the converter does
(``SBML2BSW.py:191-197,245-290``): the forward reaction, then the reverse
one with reactants and products swapped, the first named parameter being
the forward rate constant and the second the reverse one.  A reaction is
reversible when it says so (``reversible="true"``) or, with the attribute
absent (its default is true in levels 1-2), when its law names two
parameters (the converter's "assuming reversible reaction").  With
``strict=True`` a reversible law must be ``kf*[reactants] - kr*[products]``.

Species declared ``constant`` become fed species (``M_feed``, held at their
value), as ``SBML2BSW.py:302-305`` writes them: with the value 1 by default
(the converter's output), or with the species' initial amount
(``feed="initial"``).  Laws naming no parameter or more than two, events and
rules raise ``SbmlError`` naming the reaction.

    python -m lassie_gb300.sbml model.sbml out_folder [--t-end T --samples S]

writes a LASSIE input folder (``left_side``, ``right_side``, ``c_vector``,
``M_0``, ``t_vector``, and ``M_feed`` when a species is constant) for the
drop-in CLI.
"""
from __future__ import annotations

import argparse
import re
import sys
import xml.etree.ElementTree as ET
from typing import Dict, List, Optional, Tuple

import numpy as np

from .model import Model, write_folder


class SbmlError(ValueError):
    pass


def _local(tag: str) -> str:
    return tag.rsplit("}", 1)[-1]


def _children(node, name: str):
    return [c for c in node if _local(c.tag) == name]


def _child(node, name: str):
    for c in node:
        if _local(c.tag) == name:
            return c
    return None


def _ident(el) -> str:
    return el.get("id") or el.get("name") or ""


def _stoich(ref) -> int:
    s = ref.get("stoichiometry", "1")
    v = float(s)
    if v != int(v) or v < 0:
        raise SbmlError(f"non-integer stoichiometry {s!r}")
    return int(v)


# ---------------------------------------------------------------- rate laws

_TOKEN_POW = re.compile(r"^pow\(\s*([A-Za-z_][\w]*)\s*,\s*([0-9.]+)\s*\)$")


def _factors_from_formula(formula: str) -> List[Tuple[str, float]]:
    """Level-1 infix formula as a product: [(name or number text, exponent)]."""
    out = []
    for raw in formula.split("*"):
        tok = raw.strip()
        if not tok:
            raise SbmlError(f"not a product: {formula!r}")
        m = _TOKEN_POW.match(tok)
        if m:
            out.append((m.group(1), float(m.group(2))))
        elif "^" in tok:
            base, ex = tok.split("^", 1)
            out.append((base.strip(), float(ex)))
        elif re.match(r"^[A-Za-z_][\w]*$", tok) or re.match(r"^[-+0-9.eE]+$", tok):
            out.append((tok, 1.0))
        else:
            raise SbmlError(f"not a mass-action product: {formula!r}")
    return out


def _factors_from_mathml(node) -> List[Tuple[str, float]]:
    """MathML product (times of ci/cn/power) as [(name or number, exponent)]."""
    tag = _local(node.tag)
    if tag == "math":
        kids = list(node)
        if len(kids) != 1:
            raise SbmlError("kinetic law is not one expression")
        return _factors_from_mathml(kids[0])
    if tag == "ci":
        return [(node.text.strip(), 1.0)]
    if tag == "cn":
        return [(node.text.strip(), 1.0)]
    if tag == "apply":
        kids = list(node)
        op = _local(kids[0].tag)
        if op == "times":
            out = []
            for k in kids[1:]:
                out += _factors_from_mathml(k)
            return out
        if op == "power" and len(kids) == 3 and _local(kids[1].tag) == "ci" \
                and _local(kids[2].tag) == "cn":
            return [(kids[1].text.strip(), float(kids[2].text))]
    raise SbmlError("kinetic law is not a mass-action product")


def _two_sided_mathml(node):
    """``a - b`` at the top of a MathML law: (factors of a, factors of b),
    or None when the law is not a difference."""
    if _local(node.tag) == "math":
        kids = list(node)
        if len(kids) != 1:
            return None
        node = kids[0]
    if _local(node.tag) != "apply":
        return None
    kids = list(node)
    if _local(kids[0].tag) != "minus" or len(kids) != 3:
        return None
    return _factors_from_mathml(kids[1]), _factors_from_mathml(kids[2])


def _two_sided_formula(formula: str):
    """``a - b`` in a level-1 infix law (one top-level minus), or None."""
    parts = [p for p in re.split(r"(?<![eE])-", formula) if p.strip()]
    if len(parts) != 2:
        return None
    return _factors_from_formula(parts[0]), _factors_from_formula(parts[1])


def _is_number(s: str) -> bool:
    try:
        float(s)
        return True
    except ValueError:
        return False


# ------------------------------------------------------------------ reader

def _law_symbols(law) -> List[str]:
    math = _child(law, "math")
    if math is not None:
        return [e.text.strip() for e in math.iter() if _local(e.tag) == "ci" and e.text]
    return re.findall(r"[A-Za-z_][\w]*", law.get("formula") or "")


def _mass_action_rate(factors, reactants: np.ndarray, index, local) -> float:
    """k of a mass-action product whose species powers must equal
    ``reactants``."""
    rate, seen = 1.0, np.zeros(len(index), np.int64)
    for name, ex in factors:
        if name in index:
            if ex != int(ex):
                raise SbmlError(f"non-integer exponent of {name}")
            seen[index[name]] += int(ex)
        elif name in local:
            rate *= local[name] ** ex
        elif _is_number(name):
            rate *= float(name) ** ex
        else:
            raise SbmlError(f"unknown symbol {name!r}")
    if not np.array_equal(seen, reactants.astype(np.int64)):
        raise SbmlError("the rate law is not mass action in the reactants")
    return rate


def read_sbml(source: str, t: Optional[np.ndarray] = None, strict: bool = False,
              feed: str = "one") -> Model:
    """A ``Model`` from an SBML file path or SBML text.  ``t`` defaults to
    linspace(0, 10, 100).  ``feed``: the value that holds a constant species,
    "one" (LASSIE's converter) or "initial" (its initial amount)."""
    if feed not in ("one", "initial"):
        raise ValueError("feed must be 'one' or 'initial'")
    if source.lstrip().startswith("<"):
        root = ET.fromstring(source)
    else:
        root = ET.parse(source).getroot()
    model = _child(root, "model")
    if model is None:
        raise SbmlError("no <model>")
    for forbidden in ("listOfEvents", "listOfRules"):
        lst = _child(model, forbidden)
        if lst is not None and len(lst):
            raise SbmlError(f"{forbidden} are not supported")
    consts: Dict[str, float] = {}
    comps = _child(model, "listOfCompartments")
    for c in (_children(comps, "compartment") if comps is not None else []):
        consts[_ident(c)] = float(c.get("size", c.get("volume", "1")))
    params = _child(model, "listOfParameters")
    for p in (_children(params, "parameter") if params is not None else []):
        if p.get("value") is not None:
            consts[_ident(p)] = float(p.get("value"))
    species_el = _child(model, "listOfSpecies")
    if species_el is None:
        raise SbmlError("no species")
    names, x0, const = [], [], []
    for s in _children(species_el, "species"):
        names.append(_ident(s))
        v = s.get("initialConcentration", s.get("initialAmount", "0"))
        x0.append(float(v))
        const.append((s.get("constant") or "").lower() == "true")
    index = {n: i for i, n in enumerate(names)}
    level = int(root.get("level", "3"))
    comp_ids = {_ident(c) for c in (_children(comps, "compartment") if comps is not None else [])}
    rxns_el = _child(model, "listOfReactions")
    rxns = _children(rxns_el, "reaction") if rxns_el is not None else []
    N = len(names)
    left_rows, right_rows, ks = [], [], []
    for j, r in enumerate(rxns):
        rid = _ident(r) or f"#{j}"
        lrow = np.zeros(N, np.int32)
        rrow = np.zeros(N, np.int32)
        for lst, row in (("listOfReactants", lrow), ("listOfProducts", rrow)):
            el = _child(r, lst)
            for ref in (_children(el, "speciesReference") if el is not None else []):
                sp = ref.get("species")
                if sp not in index:
                    raise SbmlError(f"reaction {rid}: unknown species {sp!r}")
                row[index[sp]] += _stoich(ref)
        law = _child(r, "kineticLaw")
        if law is None:
            raise SbmlError(f"reaction {rid}: no kinetic law")
        local = dict(consts)
        for lname in ("listOfParameters", "listOfLocalParameters"):
            lp = _child(law, lname)
            for p in (list(lp) if lp is not None else []):
                if p.get("value") is not None:
                    local[_ident(p)] = float(p.get("value"))
        attr = (r.get("reversible") or "").lower()
        math = _child(law, "math")
        named = []
        for sym in _law_symbols(law):
            if sym in local and sym not in index and sym not in named and sym not in comp_ids:
                named.append(sym)
        # SBML2BSW.py:191-197: reversible when declared so, or (attribute
        # absent, default true before level 3) when the law names two
        # parameters
        reversible = attr == "true" or (attr == "" and level < 3 and len(named) == 2)
        try:
            if not strict:
                if len(named) > 2 or (len(named) == 2 and not reversible):
                    raise SbmlError(f"the kinetic law names {len(named)} parameters "
                                    f"(one rate constant expected)")
                if reversible and len(named) != 2:
                    raise SbmlError("a reversible reaction needs two rate constants "
                                    "(forward, reverse) in its kinetic law")
                if named:
                    rates = [local[n] for n in named]
                else:
                    # no parameter: a law of numbers only is read as a product
                    factors = (_factors_from_mathml(math) if math is not None
                               else _factors_from_formula(law.get("formula") or ""))
                    rates = [_mass_action_rate(factors, lrow, index, local)]
            else:
                if reversible:
                    sides = (_two_sided_mathml(math) if math is not None
                             else _two_sided_formula(law.get("formula") or ""))
                    if sides is None:
                        raise SbmlError("a reversible law must be kf*[reactants] - "
                                        "kr*[products]")
                    rates = [_mass_action_rate(sides[0], lrow, index, local),
                             _mass_action_rate(sides[1], rrow, index, local)]
                else:
                    if math is not None:
                        factors = _factors_from_mathml(math)
                    elif law.get("formula"):
                        factors = _factors_from_formula(law.get("formula"))
                    else:
                        raise SbmlError("empty kinetic law")
                    rates = [_mass_action_rate(factors, lrow, index, local)]
        except SbmlError as e:
            raise SbmlError(f"reaction {rid}: {e}") from None
        left_rows.append(lrow)
        right_rows.append(rrow)
        ks.append(rates[0])
        if reversible:
            # SBML2BSW.py:285-290: the reverse reaction follows the forward one
            left_rows.append(rrow.copy())
            right_rows.append(lrow.copy())
            ks.append(rates[1])
    R = len(left_rows)
    left = np.array(left_rows, np.int32).reshape(R, N)
    right = np.array(right_rows, np.int32).reshape(R, N)
    k = np.array(ks, np.float64)
    m = Model(left=left, right=right, k=k, x0=np.asarray(x0, np.float64),
              t=np.linspace(0.0, 10.0, 100) if t is None else np.asarray(t, np.float64))
    if any(const):
        # SBML2BSW.py:302-305: constant species are fed
        m.feed = np.array([(1.0 if feed == "one" else x0[i]) if c else 0.0
                           for i, c in enumerate(const)])
    return m


def write_sbml(m: Model, name: str = "lassie_model") -> str:
    """SBML level 1 text of ``m``: species X<i> with their initial amounts,
    irreversible reactions R<j> with local rate constants K<j> and the
    mass-action law K<j> * X<a> * ... (the layout of LASSIE's example model),
    rate constants in 17 significant digits so that read_sbml gives ``m``
    back."""
    lines = ['<?xml version="1.0" encoding="UTF-8"?>',
             '<sbml xmlns="http://www.sbml.org/sbml/level1" level="1" version="2">',
             f'\t<model name="{name}">',
             '\t<listOfCompartments>\n\t\t<compartment name="compartment01"/>\n'
             '\t</listOfCompartments>', '\t<listOfSpecies>']
    for i in range(m.n_species):
        lines.append(f'\t\t<species name="X{i}" compartment="compartment01" '
                     f'initialAmount="{m.x0[i]:.17g}" />')
    lines += ['\t</listOfSpecies>', '\t<listOfReactions>']
    for j in range(m.n_reactions):
        lines.append(f'\t\t<reaction name="R{j}" reversible="false">')
        factors = [f"K{j}"]
        for tag, row in (("listOfReactants", m.left[j]), ("listOfProducts", m.right[j])):
            nz = np.nonzero(row)[0]
            if len(nz):
                lines.append(f"\t\t\t<{tag}>")
                for i in nz:
                    lines.append(f'\t\t\t<speciesReference species="X{i}" '
                                 f'stoichiometry="{int(row[i])}"/>')
                    if tag == "listOfReactants":
                        factors += [f"X{i}"] * int(row[i])
                lines.append(f"\t\t\t</{tag}>")
        lines += [f'\t\t\t<kineticLaw formula="{"* ".join(factors)}">',
                  '\t\t\t\t<listOfParameters>',
                  f'\t\t\t\t\t<parameter name="K{j}" value="{m.k[j]:.17g}"/>',
                  '\t\t\t\t</listOfParameters>', '\t\t\t</kineticLaw>',
                  '\t\t</reaction>']
    lines += ['\t</listOfReactions>', '\t</model>', '</sbml>']
    return "\n".join(lines) + "\n"


def main(argv: Optional[List[str]] = None) -> int:
    ap = argparse.ArgumentParser(description="SBML (mass action) to a LASSIE input folder")
    ap.add_argument("sbml")
    ap.add_argument("folder")
    ap.add_argument("--t-end", type=float, default=10.0)
    ap.add_argument("--samples", type=int, default=100)
    ap.add_argument("--strict", action="store_true",
                    help="require mass-action rate laws (k = product of their constants)")
    ap.add_argument("--feed", choices=("one", "initial"), default="one",
                    help="value holding a constant species: 1 (LASSIE's converter) or its "
                         "initial amount")
    a = ap.parse_args(argv)
    try:
        m = read_sbml(a.sbml, np.linspace(0.0, a.t_end, a.samples), strict=a.strict,
                      feed=a.feed)
    except SbmlError as e:
        print(f"sbml: {e}", file=sys.stderr)
        return 2
    write_folder(m, a.folder)
    print(f"{m.n_species} species, {m.n_reactions} reactions -> {a.folder}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
