// Balanced work units of the TMA column pass (host code, no CUDA).
//
// The 2-D launch of the column pass has one CTA per (strip, work item), dispatched
// strip by strip with the items of a strip consecutive.  With `slots` CTAs resident
// at a time the launch runs in rounds; when the last round is only partly filled,
// its units are cut into shorter runs of fields so that every slot takes a share.
#pragma once

#include <algorithm>
#include <vector>

namespace fo {

struct ColUnit {
  int first;  // first position in the plan's field list
  int end;    // one past the last
  int strip;  // strip index (columns strip*W ... strip*W + W - 1)
};

// items: n_items+1 offsets into the field list (runs sharing one transfer function).
// Returns the units in dispatch order, or an empty list when the launch fits in one
// round (total <= slots) and the plain 2-D launch is kept.  An empty item (two equal
// offsets) yields no unit, so every unit holds at least one field: the persistent
// kernel issues the next unit's first strip from inside the current unit's field loop.
inline std::vector<ColUnit> balanced_col_units(const std::vector<int>& items, int strips, int slots) {
  std::vector<ColUnit> units;
  const int n_items = (int)items.size() - 1;
  if (n_items < 1 || strips < 1 || slots < 1) return units;
  for (int st = 0; st < strips; ++st)
    for (int i = 0; i < n_items; ++i)
      if (items[i + 1] > items[i]) units.push_back(ColUnit{items[i], items[i + 1], st});
  const int total = (int)units.size();
  if (total <= slots) return {};
  const int tail = total % slots;
  if (tail != 0) {
    std::vector<ColUnit> last(units.end() - tail, units.end());
    units.resize(total - tail);
    const int pieces = std::max(1, slots / tail);
    for (const ColUnit& u : last) {
      const int len = u.end - u.first;
      const int k = std::max(1, std::min(pieces, len));
      for (int j = 0; j < k; ++j)
        units.push_back(ColUnit{u.first + j * len / k, u.first + (j + 1) * len / k, u.strip});
    }
  }
  return units;
}

}  // namespace fo
