"""Where the reference's sources are read from (test infrastructure).

The checker build (oracle/ref/build_ref.py), the golden-fixture script and
the tests that read the reference's shipped case files take the reference
root from the SPHDEM_REFERENCE_ROOT environment variable, defaulting to the
read-only checkout this recipe was written against.  Where the directory is
absent, those steps are skipped.
"""
import os

REF_ROOT = os.environ.get("SPHDEM_REFERENCE_ROOT", "/root/reference")


def present() -> bool:
    return os.path.isdir(REF_ROOT)
