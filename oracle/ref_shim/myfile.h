// Stand-in for msfitslib's MyFile: the oracle build never reads metadata files.
#pragma once
struct MyFile { static bool DoesFileExist(const char *) { return false; } };
