/* Environment.cpp:7 includes the application header; nothing from it is used
   by the simulator, so the oracle build gives it an empty file. */
#pragma once
