#!/usr/bin/env bash
# Builds oracle/liboracle.so, the C restatement used as the CPU checker.
# -ffp-contract=off: identical tree arithmetic on x86-64 and AArch64 hosts.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared -std=c11 -D_DEFAULT_SOURCE \
    -o "$HERE/liboracle.so" "$HERE/oracle.c" -lm
