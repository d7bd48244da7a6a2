"""Builds the sm_103a library (tapkee_gb300/_lib/libtapkee_gb300.so, with nvcc)
before the package files are copied, so that a wheel or an install carries it."""
import importlib.util
import os

from setuptools import setup
from setuptools.command.build_py import build_py

HERE = os.path.dirname(os.path.abspath(__file__))


class BuildWithLibrary(build_py):
    def run(self):
        spec = importlib.util.spec_from_file_location("tk_build", os.path.join(HERE, "tapkee_gb300", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
        super().run()


setup(cmdclass={"build_py": BuildWithLibrary})
