// Stand-in for the reference's core/Logger.h (test oracle build only).
#pragma once
