// Empty stand-in: the compiled reference math files use no OpenGL.
#pragma once
