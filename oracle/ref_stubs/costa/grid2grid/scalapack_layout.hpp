// Stand-in for the one COSTA type named by the reference's scalapack.hpp.
#pragma once
namespace costa {
namespace scalapack {
enum class ordering { row_major, column_major };
}
}  // namespace costa
