// netscience.h names tinyxml2; the oracle's reference build does not read XML
#pragma once
namespace tinyxml2 {}
