// Empty stand-in so the reference kernel headers compile without their GUI/graphics dependencies.
#pragma once
