"""Where the tests find the reference tree when it is present (it is read only: golden runs of its
kernel, its data files). FLYBRAIN_REFERENCE overrides the location; tests that need it skip when
it is absent."""
import os

REFERENCE = os.environ.get("FLYBRAIN_REFERENCE", "/root/reference")
REF_DATA = os.path.join(REFERENCE, "public", "data")
REF_LIF_C = os.path.join(REFERENCE, "src", "wasm", "lif.c")
