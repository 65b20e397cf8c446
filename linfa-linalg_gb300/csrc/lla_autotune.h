// lla_autotune.h -- the autotune cache shared by the batched plans and the
// refined solve: one line per key, "key a b", in LLA_AUTOTUNE_CACHE (default
// ~/.cache/lla_gb300_autotune.txt).  The file is read once per path and then
// answered from memory; a store appends to the file, and the last line for a
// key wins.
#pragma once

#include <string>

namespace lla {

bool autotune_lookup(const std::string &key, int &a, int &b);
void autotune_store(const std::string &key, int a, int b);

}  // namespace lla
