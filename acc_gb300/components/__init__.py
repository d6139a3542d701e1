"""Components with the reference's module paths and class names
(mcvine.acc.components.*)."""
