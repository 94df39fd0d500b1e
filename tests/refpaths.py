"""Where the tests find the reference tree when it is present (it is read only: its data files).
The location comes from FLYBRAIN_REFERENCE alone; tests that need the tree skip when it is unset.
Tests of the reference kernel itself use its native build (oracle/_ref), made by oracle/Makefile."""
import os

REFERENCE = os.environ.get("FLYBRAIN_REFERENCE", "")
REF_DATA = os.path.join(REFERENCE, "public", "data") if REFERENCE else ""
