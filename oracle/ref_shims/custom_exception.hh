// Stand-in for Backend/includes/tools/exception/custom_exception.hh in the comparison build:
// std::exception has no const char* constructor outside MSVC, so the message is kept in a
// std::runtime_error base.
#pragma once

#include <stdexcept>
#include <string>

namespace holovibes
{
class CustomException : public std::runtime_error
{
  public:
    CustomException(const std::string& msg)
        : std::runtime_error(msg)
    {
    }
    CustomException(const std::string& msg, const int, const char*)
        : std::runtime_error(msg)
    {
    }
};
} // namespace holovibes
