// Test-only stand-in for boost::shared_ptr (std::shared_ptr underneath).
#pragma once
#include <memory>
namespace boost
{
using std::shared_ptr;
}
