#!/bin/sh
# TEST INFRASTRUCTURE ONLY.
# Builds the reference library from its own sources where they lie into
# oracle/_ref/libref.so (git-ignored), for pinning the oracle and generating
# tests/golden/.  The reference's kernels are x86-64 NASM; nasm is not in the
# image, so the .asm is translated mechanically to GNU-as Intel syntax into
# oracle/_ref/ and assembled there.  Nothing from the reference is committed.
# Skips (exit 0) on non-x86-64 hosts or when the reference is absent.
set -e
REF=${NN_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ "$(uname -m)" != "x86_64" ] || [ ! -f "$REF/asmLinux.asm" ]; then
  echo "build_ref: reference not buildable here (needs x86-64 and $REF)"; exit 0
fi
mkdir -p "$OUT"
{
  echo '.intel_syntax noprefix'
  sed -e 's/;/#/' \
      -e 's/^default rel//' \
      -e 's/^extern memcpy//' \
      -e 's/^section \.note\.GNU-stack.*/.section .note.GNU-stack,"",@progbits/' \
      -e 's/^section \.text/.text/' \
      -e 's/^global /.globl /' \
      -e 's/qword \[/qword ptr [/g' \
      -e 's/call memcpy wrt \.\.plt/call memcpy@PLT/' \
      -e 's/\b\([0-9][0-9a-fA-F]*\)h\b/0x\1/g' \
      "$REF/asmLinux.asm"
  echo
} > "$OUT/asmLinux.s"
as "$OUT/asmLinux.s" -o "$OUT/asmLinux.o"
g++ -O2 -std=c++20 -fPIC -shared -w -I"$REF" "$HERE/ref_shim.cpp" "$OUT/asmLinux.o" -o "$OUT/libref.so"
echo "build_ref: built $OUT/libref.so"
