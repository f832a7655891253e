"""Locations of the in-tree shared libraries."""
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG_DIR, "_lib")
CSRC_DIR = os.path.join(PKG_DIR, "csrc")
REPO_DIR = os.path.dirname(PKG_DIR)
INCLUDE_DIR = os.path.join(REPO_DIR, "include")


def lib_path(name: str) -> str:
    return os.path.join(LIB_DIR, name)
