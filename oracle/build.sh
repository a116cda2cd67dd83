#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/build/liboracle.so.
# -ffp-contract=off keeps every float32 a*b+c two roundings, as the
# reference's Go evaluates it on amd64.
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/build"
${CXX:-g++} -O2 -std=c++17 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread \
    -o "$here/build/liboracle.so" "$here/oracle.cpp" "$here/adjoint.cpp"
