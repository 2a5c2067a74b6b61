// mechanism.H — test stand-in: NUM_SPECIES of the test's synthetic mechanism.
#pragma once
#include "mechanism_table.H"
