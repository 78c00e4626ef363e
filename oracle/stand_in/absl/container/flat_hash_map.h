// Stand-in for absl/container/flat_hash_map.h: the reference includes it but
// uses nothing from it.
#pragma once
