#pragma once
#include <boost/signals2.hpp>
