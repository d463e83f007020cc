// Declarations the reference's headers name from AntTweakBar (GUI library,
// not part of the pin); nothing here is called.
#pragma once
typedef struct CTwBar TwBar;
const char* TwGetLastError();
