// Minimal fmt colour subset — TEST INFRASTRUCTURE (the reference's console output headers include it).
#pragma once
#include "core.h"
