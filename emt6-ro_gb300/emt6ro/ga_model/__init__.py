from .model import EMT6RoModel
