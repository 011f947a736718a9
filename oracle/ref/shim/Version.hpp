// Version header normally written by the reference's CMake configure step.
#pragma once
#include <string_view>
namespace OpFlow::internal {
inline constexpr auto OPFLOW_VERSION_STRING = std::string_view {"0.2.7"};
}
