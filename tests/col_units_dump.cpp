// Prints the balanced column work units for one configuration (test helper).
// usage: col_units_dump strips slots item_offset0 item_offset1 ...
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fo_units.h"

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  const int strips = std::atoi(argv[1]), slots = std::atoi(argv[2]);
  std::vector<int> items;
  for (int i = 3; i < argc; ++i) items.push_back(std::atoi(argv[i]));
  for (const fo::ColUnit& u : fo::balanced_col_units(items, strips, slots)) std::printf("%d %d %d\n", u.first, u.end, u.strip);
  return 0;
}
