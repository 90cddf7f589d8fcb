#pragma once
#define GSL_SUCCESS 0
#define GSL_EDOM 1
