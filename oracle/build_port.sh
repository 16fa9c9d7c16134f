#!/usr/bin/env bash
# Test infrastructure: build the oracle restatement oracle/sfci_port.cpp into
# oracle/_port/libsfci_port.so (portable flags: it is rebuilt on every host).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_port"
# built under a temporary name and renamed, so a process that has the old
# library loaded keeps its mapping
g++ -std=c++17 -O2 -fopenmp -fPIC -shared -Wall -Wno-unused-function \
    "$HERE/sfci_port.cpp" -o "$HERE/_port/libsfci_port.so.tmp.$$"
mv -f "$HERE/_port/libsfci_port.so.tmp.$$" "$HERE/_port/libsfci_port.so"
echo "built $HERE/_port/libsfci_port.so"
