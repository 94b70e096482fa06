"""Legacy text writers (src/utils.cpp:211-236): the Python ones and the C++
facade's write the same bytes, in the C++ stream's default formatting."""
import io
import os
import subprocess

import numpy as np

from jetshow_gb300.textio import write_2dvector, write_vector

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CPP = r'''
#include <iostream>
#include <limits>
#include "jetshow.hpp"
int main() {
  std::vector<std::vector<double>> img = {{1.0, 2.5e-7, -3.0}, {1234567.0, 0.0, 1e300},
                                          {std::numeric_limits<double>::infinity(), -0.0, 0.125}};
  jetshow::write_2dvector(std::cout, img, 2.0);
  jetshow::write_vector(std::cout, std::vector<double>{3.0, 1e-20, 42.0}, 3.0);
  return 0;
}
'''


def expected():
    img = [[1.0, 2.5e-7, -3.0], [1234567.0, 0.0, 1e300], [float("inf"), -0.0, 0.125]]
    f = io.StringIO()
    write_2dvector(f, img, 2.0)
    write_vector(f, [3.0, 1e-20, 42.0], 3.0)
    return f.getvalue()


def test_python_writers_format():
    f = io.StringIO()
    write_2dvector(f, np.array([[1.0, 2.0], [3.0, 4.5]]), 2.0)
    assert f.getvalue() == "0.5 1 \n1.5 2.25 \n"
    f = io.StringIO()
    write_vector(f, [1e-7, 123456789.0])
    assert f.getvalue() == "1e-07 \n1.23457e+08 \n"


def test_cpp_and_python_writers_agree(tmp_path):
    src = tmp_path / "w.cpp"
    src.write_text(CPP)
    exe = tmp_path / "w"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    assert out == expected()
