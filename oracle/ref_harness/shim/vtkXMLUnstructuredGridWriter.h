/* Empty stand-in: the reference includes this VTK header only for its file writers, which the oracle build replaces. */
#pragma once
