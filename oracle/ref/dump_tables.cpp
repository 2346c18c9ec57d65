// Dumps the reference's marching-cubes tables (src/tables.h) into a small binary
// fixture so the tests can check this project's own table copy against the
// reference's data.  Compiled and run by oracle/ref/build_ref.py at fixture
// generation time; never part of the product.
#include <cstdio>
#include <cstdint>
#include <sys/types.h>
#include REF_TABLES_H

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  FILE* f = std::fopen(argv[1], "wb");
  if (!f) return 1;
  // layout: u16 edgeTable[256], u8 triTable[256][16], u8 numVertsTable[256]
  for (int i = 0; i < 256; ++i) { uint16_t v = (uint16_t)edgeTable[i]; std::fwrite(&v, 2, 1, f); }
  for (int i = 0; i < 256; ++i)
    for (int j = 0; j < 16; ++j) { uint8_t v = (uint8_t)triTable[i][j]; std::fwrite(&v, 1, 1, f); }
  for (int i = 0; i < 256; ++i) { uint8_t v = (uint8_t)numVertsTable[i]; std::fwrite(&v, 1, 1, f); }
  std::fclose(f);
  return 0;
}
