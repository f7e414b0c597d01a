#pragma once
#include <boost/iostreams/filtering_streambuf.hpp>
