/* MSVC <intrin.h> stand-in for the reference build on Linux/x86 (oracle recipe only). */
#pragma once
#include <x86intrin.h>
