#!/bin/sh
# Compile the reference's CPU draw path from its own sources (unmodified, read
# in place) plus this project's glue into one shared library.  TEST INFRASTRUCTURE.
#   build_ref.sh REFERENCE REPO OBJDIR EXTRA_FLAGS OUTPUT
set -e
REF="$1"; REPO="$2"; OBJ="$3"; EXTRA="$4"; OUT="$5"
mkdir -p "$OBJ"
CXX="g++ -std=c++17 -O2 -fPIC -ffp-contract=off -fno-strict-aliasing -w $EXTRA"
REFF="-DMICROPROFILE_ENABLED=0 -include $REPO/oracle/ref/shim.h -I$REF"
pids=""
for f in precompiled rasterizer texture_sampling cmd_exec cmd_record cmd_alloc memory buffers \
         images descriptors renderpass shaders icd_stubs icd_interface query stats; do
  $CXX $REFF -c "$REF/$f.cpp" -o "$OBJ/$f.o" & pids="$pids $!"
done
gcc -std=c99 -O2 -fPIC -ffp-contract=off -w -include "$REPO/oracle/ref/shim.h" -c "$REF/3rdparty/decompress.c" -o "$OBJ/decompress.o" & pids="$pids $!"
$CXX $REFF -I"$REPO/include" -c "$REPO/oracle/ref/glue.cpp" -o "$OBJ/glue.o" & pids="$pids $!"
$CXX -DVISOR_DRIVER_KHRONOS_HEADER -I"$REF" -I"$REPO/include" -c "$REPO/visor_gb300/csrc/scene/driver.cpp" -o "$OBJ/driver.o" & pids="$pids $!"
gcc -std=c11 -O2 -fPIC -ffp-contract=off -I"$REPO/include" -c "$REPO/visor_gb300/csrc/scene/scene.c" -o "$OBJ/scene.o" & pids="$pids $!"
gcc -std=c11 -O2 -fPIC -ffp-contract=off -I"$REPO/include" -c "$REPO/visor_gb300/csrc/scene/spirv_emit.c" -o "$OBJ/spirv_emit.o" & pids="$pids $!"
for p in $pids; do wait $p; done
g++ -shared -o "$OUT" "$OBJ"/*.o -lpthread -lm
