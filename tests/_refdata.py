"""Where the reference project's data files are, for the CPU tests that read
them: GPUBOSCIA_REFERENCE when set, else the root that oracle/build.sh
recorded when it compiled the reference's CPU functions. None when neither
exists (the tests that need the files then skip)."""
import os
import pathlib

ROOT = pathlib.Path(__file__).resolve().parent.parent


def reference_root():
    env = os.environ.get("GPUBOSCIA_REFERENCE")
    if env:
        return pathlib.Path(env)
    rec = ROOT / "oracle" / "_ref" / "reference_root.txt"
    if rec.is_file():
        return pathlib.Path(rec.read_text().strip())
    return None


def reference_path(*parts):
    """A path inside the reference tree, or a path that does not exist."""
    r = reference_root()
    return r.joinpath(*parts) if r is not None else ROOT / "oracle" / "_ref" / "absent" / pathlib.Path(*parts)
