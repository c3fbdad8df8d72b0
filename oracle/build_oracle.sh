#!/bin/sh
# Builds the CPU oracle (oracle/kpt_oracle.cpp, IEEE single precision, and
# oracle/adjoint_oracle.cpp, double precision) into oracle/libkpt_oracle.so,
# without contraction, so that x86-64 and aarch64 builds compute the same
# values.
set -e
here=$(cd "$(dirname "$0")" && pwd)
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -fno-fast-math \
    "$here/kpt_oracle.cpp" "$here/adjoint_oracle.cpp" -o "$here/libkpt_oracle.so" -lpthread
echo "built $here/libkpt_oracle.so"
