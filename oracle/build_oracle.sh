#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure only) into oracle/liboracle.so.
# -ffp-contract=off keeps every product and sum separately rounded, as in the
# Rust reference; -fopenmp is used only by the multi-threaded CPU baseline.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -fopenmp \
    -o "$here/liboracle.so" "$here/axia_oracle.cpp"
