// Stand-in for the libconfig C header (the reference includes it but uses only the C++ API).
#pragma once
