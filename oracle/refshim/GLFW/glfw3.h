// Stand-in declaring the two GLFW names that src/base/utility.h mentions.
#pragma once
typedef struct GLFWwindow GLFWwindow;
#define GLFW_KEY_LAST 348
