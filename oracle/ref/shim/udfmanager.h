/*
 * Stand-in for OCTA's udfmanager.h (libplatform is not available). The
 * oracle build never parses UDF files: the harness sets the reference's
 * global parameters directly. Only the type names used in declarations are
 * provided. TEST INFRASTRUCTURE ONLY.
 */
#ifndef ICEP_ORACLE_UDFMANAGER_STUB_H
#define ICEP_ORACLE_UDFMANAGER_STUB_H
#include <string>
using namespace std; /* the OCTA header exposes std names unqualified */
class UDFManager;
class Location;
#endif
