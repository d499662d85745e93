"""Where the reference tree (ls1-mardyn sources) lives, for the scripts and
tests that read it: $LS1_REFERENCE, else a checkout named ``reference`` beside
this repository.  Test infrastructure only; nothing on the product path
reads the reference."""
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_tree() -> str:
    return os.environ.get("LS1_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
