#!/usr/bin/env bash
# Writes the 1024 in-cell positions of the reference's shape unit test
# (share/picongpu/unit/shape.cpp:176-185: std::mt19937 mt(42.0),
# std::uniform_real_distribution<> dist(0.0, 1.0), stored as float_X = float)
# to shape_positions_mt19937_42.f32 (raw little-endian float32).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
tmp="$(mktemp -d)"
cat > "$tmp/gen.cpp" <<'CPP'
#include <cstdio>
#include <random>
int main()
{
    std::mt19937 mt(42.0);
    std::uniform_real_distribution<> dist(0.0, 1.0);
    for(int i = 0; i < 1024; ++i)
    {
        float v = static_cast<float>(dist(mt));
        std::fwrite(&v, sizeof(float), 1, stdout);
    }
    return 0;
}
CPP
g++ -O1 -o "$tmp/gen" "$tmp/gen.cpp"
"$tmp/gen" > "$here/shape_positions_mt19937_42.f32"
rm -rf "$tmp"
