// Project-written stand-in: everything lives in owl/owl.h.
#pragma once
#include <owl/owl.h>
