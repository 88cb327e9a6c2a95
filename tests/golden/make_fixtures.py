"""Copy the reference's driver configuration templates into tests/golden/.

The reference ships two libconfig files next to its sources,
parameters_template.cfg (the driver_mgmc run configuration,
src/auxilliary/parameters.cc:259-350 reads it) and measurements_template.cfg
(the measurement file it names).  They are the only golden inputs the
reference has for configuration ingestion; tests/test_config.py parses the
copies made here.  Run from the repository root with the reference checkout
given by MGMC_REFERENCE_ROOT (default: the directory `reference` next to the
repository):

    python tests/golden/make_fixtures.py
"""
import os
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("MGMC_REFERENCE_ROOT", os.path.join(os.path.dirname(REPO), "reference"))

FILES = ("parameters_template.cfg", "measurements_template.cfg")


def main():
    for name in FILES:
        src = os.path.join(REF, name)
        shutil.copyfile(src, os.path.join(HERE, name))
        print(f"copied {src}")


if __name__ == "__main__":
    main()
