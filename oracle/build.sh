#!/bin/sh
# Build the CPU oracle (test infrastructure; see somref.cpp).
# -ffp-contract=off: no fused multiply-add, so x86_64 and aarch64 hosts round identically.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -fPIC -shared -o "$HERE/libsomref.so" "$HERE/somref.cpp"
