"""Where the in-tree build puts each shared library."""
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
SIH_DIR = os.path.dirname(PKG_DIR)  # sih-26_gb300/
REPO_DIR = os.path.dirname(SIH_DIR)
CSRC_DIR = os.path.join(SIH_DIR, "csrc")
LPGEN_DIR = os.path.join(SIH_DIR, "lpgen")
INCLUDE_DIR = os.path.join(REPO_DIR, "include")

ENGINE_LIB = os.path.join(SIH_DIR, "lib", "libsankhya_gb300.so")
LPGEN_LIB = os.path.join(SIH_DIR, "lib", "liblpgen.so")
