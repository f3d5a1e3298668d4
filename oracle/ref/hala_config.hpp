/* Configuration header for building the reference's CPU path without its CMake (test infra). */
#ifndef __HALA_CONFIG_HPP
#define __HALA_CONFIG_HPP
#define HALA_LICENSE "BSD-3-Clause"
#define HALA_VERSION_MAJOR 1
#define HALA_VERSION_MINOR 1
#define HALA_VERSION_PATCH 0
#endif
