// types.h -- scalar types of the host mirror, as in common/include/common/types.h.
#pragma once

#include <cstdint>

namespace physicore {

using real_t = double;
using index_t = std::uint64_t;
using sindex_t = std::int64_t;

} // namespace physicore
