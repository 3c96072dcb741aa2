#!/usr/bin/env bash
# Builds the reference renderer's own code (drcd1/cpp-pt, header-only C++) as a
# shared library for the oracle harness.  Test infrastructure only.
#
#   oracle/build_ref.sh [REFERENCE_ROOT]   (default: $CPPPT_REFERENCE_ROOT, else /root/reference)
#
# Step 1 (only where REFERENCE_ROOT exists): copy REFERENCE_ROOT/src and the
#   vendored stb headers into oracle/_ref/src and apply the compat patches below
#   (the reference is written for MSVC; g++ rejects six constructs).  Each patch
#   is one sed expression; none changes arithmetic.
# Step 2 (wherever oracle/_ref/src exists, e.g. after the copy travelled to
#   another machine): compile oracle/ref_harness.cpp against that copy into
#   oracle/_ref/libref_harness.so with -O2 -fopenmp -ffp-contract=off.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${CPPPT_REFERENCE_ROOT:-/root/reference}}"
OUT="$HERE/_ref"
mkdir -p "$OUT"
if [ -d "$REF/src" ]; then
  rm -rf "$OUT/src"
  mkdir -p "$OUT/src"
  cp -r "$REF/src/." "$OUT/src/"
  cp -r "$REF/third-party/stb" "$OUT/src/stb"
  S="$OUT/src"
  # (1) math/math.h:33  Vector4::operator-() names an undeclared 'a'
  sed -i 's/return {-x,-y,-z,-a\.w};/return {-x,-y,-z,-w};/' "$S/math/math.h"
  # (2) image/rgb_image.h:33  functional cast with a two-word type name
  sed -i 's/\*pix = unsigned char(unsigned int(a\*255\.0));/*pix = (unsigned char)((unsigned int)(a*255.0));/' "$S/image/rgb_image.h"
  # (3) math/sampler.h:61  std::modff is not declared by libstdc++
  sed -i 's/std::modff(/modff(/' "$S/math/sampler.h"
  # (4) primitive/bvh.h:18  constructor must take the child pointers by rvalue
  sed -i 's/BVHNode(std::unique_ptr<Primitive>& right, std::unique_ptr<Primitive>& left, AABB& aabb)/BVHNode(std::unique_ptr<Primitive>\&\& right, std::unique_ptr<Primitive>\&\& left, AABB\& aabb)/' "$S/primitive/bvh.h"
  # (5) renderer/pathtracerMIS.h:36  hard-coded 32 bounces -> harness setting
  sed -i 's/for(int i = 0; i<32; i++){/for(int i = 0; i<cpppt_harness_max_depth; i++){/' "$S/renderer/pathtracerMIS.h"
  # (6) renderer/pathtracerMIS.h:143-144  column seed offset (independent replicas) and quiet progress
  sed -i 's/RandomSampler s(i);/RandomSampler s(i + cpppt_harness_seed_offset);/; s/if(i%50==0)/if(cpppt_harness_verbose \&\& i%50==0)/' "$S/renderer/pathtracerMIS.h"
  # (7) renderer/ppg.h: same two settings for the SD-tree guided comparison path
  sed -i 's/RandomSampler s(i);/RandomSampler s(i + cpppt_harness_seed_offset);/' "$S/renderer/ppg.h" || true
  # (8) renderer/pure_pt.h, renderer/pathtracer.h: the bounce limit, seed offset and quiet progress
  #     of (5)-(6) for the pure-PT and PT+NEE integrators
  for f in pure_pt.h pathtracer.h; do
    sed -i 's/for(int i = 0; i<32; i++){/for(int i = 0; i<cpppt_harness_max_depth; i++){/; s/RandomSampler s(i);/RandomSampler s(i + cpppt_harness_seed_offset);/; s/if(i%50==0)/if(cpppt_harness_verbose \&\& i%50==0)/' "$S/renderer/$f"
    grep -q 'cpppt_harness_max_depth' "$S/renderer/$f"
  done
  # (9) texture/image_texture.h:21  ImageTexture::filtering is never initialised (the image-texture
  #     path reads an indeterminate value); the harness pins it to the bilinear branch, which the
  #     GPU texture sampler implements
  sed -i 's/^    Filtering filtering;/    Filtering filtering = BILINEAR;/' "$S/texture/image_texture.h"
  grep -q 'Filtering filtering = BILINEAR;' "$S/texture/image_texture.h"
  grep -q 'cpppt_harness_max_depth' "$S/renderer/pathtracerMIS.h"
  grep -q 'unique_ptr<Primitive>&& right' "$S/primitive/bvh.h"
fi
if [ ! -d "$OUT/src" ]; then
  echo "build_ref: no reference sources (neither $REF/src nor $OUT/src)" >&2
  exit 3
fi
CXX="${CXX:-g++}"
"$CXX" -std=c++17 -O2 -fopenmp -ffp-contract=off -fPIC -shared -fpermissive -w \
  -include memory -include cmath -include math.h -include fstream \
  -I"$OUT/src" -o "$OUT/libref_harness.so" "$HERE/ref_harness.cpp"
echo "build_ref: built $OUT/libref_harness.so"
