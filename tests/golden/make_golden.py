"""Regenerates the golden fixtures in this folder from the reference's own test data.

Reads ``tests/resources/CLASS_data.json``,
``tests/resources/RECFAST_DISCO_EB_data.json`` and
``tests/resources/RECFAST_CLASS_data.json`` of the reference checkout
(path given as the first argument) and writes trimmed copies here, so the
tests never need the reference at run time:

* ``class_pkbc_a0p01.json``: all 616 (k, P_bc) pairs, a = 0.01, CLASS,
  the fixture of ``tests/test_perturbations.py:62-64,140-142``;
* ``recfast_xe_v010.json``: every 3rd (a, x_e) pair of the DISCO-EB v0.1.0
  RECFAST baseline, the fixture of ``tests/test_background.py:71-75``;
* ``recfast_xe_class.json``: every 10th (a, x_e) pair of
  ``tests/resources/RECFAST_CLASS_data.json`` (CLASS's RECFAST for the same
  cosmology; shipped with the reference, loaded by none of its tests).

Usage: python tests/golden/make_golden.py <reference-root>
"""
import json
import os
import sys

here = os.path.dirname(os.path.abspath(__file__))
root = sys.argv[1]
res = os.path.join(root, "tests", "resources")
cls = json.load(open(os.path.join(res, "CLASS_data.json")))
json.dump({"k": cls["k"], "Pkbc": cls["Pkbc"], "aexp": 0.01,
           "source": "reference tests/resources/CLASS_data.json"},
          open(os.path.join(here, "class_pkbc_a0p01.json"), "w"))
rf = json.load(open(os.path.join(res, "RECFAST_DISCO_EB_data.json")))
json.dump({"a": rf["a"][::3], "xe": rf["xe"][::3],
           "source": "reference tests/resources/RECFAST_DISCO_EB_data.json (every 3rd pair)"},
          open(os.path.join(here, "recfast_xe_v010.json"), "w"))
rc = json.load(open(os.path.join(res, "RECFAST_CLASS_data.json")))
json.dump({"a": rc["a"][::10], "xe": rc["xe"][::10],
           "source": "reference tests/resources/RECFAST_CLASS_data.json (every 10th pair)"},
          open(os.path.join(here, "recfast_xe_class.json"), "w"))
