"""Writes tests/golden/published.json.

The values are transcribed by hand from the reference's README (the output of
its bench/bench.py on the machine it names, README.md:274-321, and the README
usage example, README.md:91-94).  They are the reference's own published known
answers for the Krylov path; nothing here is computed.
"""
import json
import os

PUBLISHED = {
    "cg+none": {"32": 113, "64": 225, "128": 434},
    "gmres+none": {"32": 232, "64": 626, "128": 2000},
    "fgmres+none": {"32": 232, "64": 626, "128": 2000},
    "bcgs+none": {"32": 85, "64": 162, "128": 316},
    "cg+ilu": {"32": 40, "64": 77, "128": 146},
    "cg+icc": {"32": 40, "64": 77, "128": 146},
    "gmres+jacobi": {"32": 232, "64": 626},
}

if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "published.json")
    with open(path) as f:
        doc = json.load(f)
    doc["iterations"] = PUBLISHED
    with open(path, "w") as f:
        json.dump(doc, f, indent=2)
