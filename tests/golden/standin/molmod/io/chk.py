"""molmod.io.chk stand-in: the product's CHK reader/writer."""
from micmec_gb300.chk import load_chk, dump_chk  # noqa: F401
